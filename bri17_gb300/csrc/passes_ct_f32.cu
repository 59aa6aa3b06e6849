// Compile-time-length power-of-two passes, FP32 instances, and the FP32
// TMA-staged axis-0 stiffness pass (none at FP64: that pass is bound by the
// FP64 pipe, not by memory).
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT_INSTANTIATE(float)

bool ct_axis0_stiffness_tma_f32(int n0, bool keep, cplx<float>* X, int64_t P, int64_t cstride,
                                int64_t bstride, int batch, const FusedParams<float>& fp,
                                BatchMask mask, cudaStream_t st) {
  return ct_axis0_stiffness_tma<float>(n0, keep, X, P, cstride, bstride, batch, fp, mask, st);
}

void ct_set_smem_attrs_tma_f32(size_t max_smem) { ct_set_smem_attrs_tma<float>(max_smem); }

cudaError_t tma_set_wait_limit_f32(uint64_t ns) {
  const unsigned long long v = ns;
  return cudaMemcpyToSymbol(g_tma_wait_limit_ns, &v, sizeof(v));
}

cudaError_t tma_wait_timeouts_f32(int* count) {
  int n = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&n, g_tma_timeouts, sizeof(int));
  if (e == cudaSuccess && n) {
    const int zero = 0;
    e = cudaMemcpyToSymbol(g_tma_timeouts, &zero, sizeof(int));
  }
  *count = n;
  return e;
}

}  // namespace bri17gb
