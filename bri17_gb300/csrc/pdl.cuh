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

#include <utility>

namespace bri17gb {

__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
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
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace bri17gb
