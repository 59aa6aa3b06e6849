// pdl.cuh -- programmatic dependent launch for the operator's passes.
//
// The passes of one operator application are launched back to back on one
// stream, each with cudaLaunchAttributeProgrammaticStreamSerialization.  A
// pass signals `griddepcontrol.launch_dependents` at its start, so the next
// pass is launched as soon as every CTA of this one is resident; the next
// pass then loads its constant tables into shared memory and executes
// `griddepcontrol.wait` -- which returns when the previous grid has
// completed and its memory is visible -- before it reads or writes any
// field.  The launch latency and table set-up of each pass overlap the tail
// of the previous one.  Without the attribute both instructions are no-ops.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <utility>

namespace bri17gb {

__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Which pass sequences are chained.  Measured on the GB300 (FP32 operator,
// five passes): chaining hides the launch latency of short passes (128^3:
// 0.098 -> 0.061 ms per application; FP64 and float pairs at 128^3 gain
// 1.5% and 4.5%), but slows the passes over large spectra (256^3: 0.460 ->
// 0.515 ms; 512x512x128: 0.985 -> 1.184 ms, the passes themselves running
// slower).  So a sequence is chained when each of its passes moves at most
// kPdlMaxEntries complex spectrum entries (all components and batch
// entries).  BRI17_PDL=0 or =1 forces plain or chained launches (for
// measurements).
constexpr int64_t kPdlMaxEntries = int64_t(8) << 20;

inline int pdl_env_mode() {
  static const int mode = [] {
    const char* e = getenv("BRI17_PDL");
    if (!e) return -1;
    return strcmp(e, "0") == 0 ? 0 : strcmp(e, "1") == 0 ? 1 : -1;
  }();
  return mode;
}

inline bool pdl_for_entries(int64_t entries) {
  const int m = pdl_env_mode();
  return m >= 0 ? m == 1 : entries <= kPdlMaxEntries;
}

// The calling thread's choice for the launches it makes (set by PdlScope
// around one pass sequence).
inline bool& pdl_thread_flag() {
  thread_local bool on = true;
  return on;
}

struct PdlScope {
  bool prev;
  explicit PdlScope(bool on) : prev(pdl_thread_flag()) { pdl_thread_flag() = on; }
  ~PdlScope() { pdl_thread_flag() = prev; }
  PdlScope(const PdlScope&) = delete;
  PdlScope& operator=(const PdlScope&) = delete;
};

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_thread_flag() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace bri17gb
