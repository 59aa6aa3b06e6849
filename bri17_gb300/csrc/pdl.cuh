// pdl.cuh -- programmatic dependent launch for the operator's passes.
//
// The passes of one operator application are launched back to back on one
// stream, each with cudaLaunchAttributeProgrammaticStreamSerialization, so
// the next pass's launch is prepared while the previous one runs.  The next
// pass loads its constant tables into shared memory and then executes
// `griddepcontrol.wait` -- which returns when the previous grid has
// completed and its memory is visible -- before it reads or writes any
// field.  When the previous pass triggers early (`launch_dependents` at the
// start of its CTAs, FP64 passes; see below), the next pass's CTAs start
// while the previous pass's last CTAs still run; otherwise as those exit.
// Without the attribute both instructions are no-ops.
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <utility>

namespace bri17gb {

// Early trigger, for FP64 passes only.  With it a pass lets the next one
// launch as soon as all of its CTAs are running, so the next pass's CTAs
// become resident during this pass's tail.  Without it the next pass
// launches as this pass's CTAs exit (still ahead of a plain stream launch).
// Measured on the GB300, the early trigger pays for the FP64 passes, which
// are bound by the FP64 pipe (128^3: 0.928 -> 0.925 ms per application).
// For the memory-bound FP32 passes and the float-pair passes it slowed the
// tails: FP32 256^3 0.515 ms against 0.446 ms without it, 512x512x128
// 1.187 against 0.974 ms; float pairs at 128^3 25.6 against 25.8 GDoF/s.
template <typename T>
__device__ __forceinline__ void pdl_launch_dependents() {
  if constexpr (std::is_same<T, double>::value)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// BRI17_PDL=0 launches the passes without the attribute (plain stream
// order; for measurements).
inline bool pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("BRI17_PDL");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on;
}

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
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace bri17gb
