// Float-pair (df64.cuh) instances of the axis-0 stiffness pass: the
// shared-memory staged and TMA-staged forms (the register-resident form
// needs more than 255 registers in float pairs).  The other float-pair
// passes are in passes_df_rows.cu and passes_df_c2c.cu, so the three
// translation units compile in parallel.
#include "passes_ct.cuh"

namespace bri17gb {

template bool ct_axis0_stiffness_staged<df64, 2>(int, cplx<df64>*, int64_t, int64_t, int64_t,
                                                 int, const FusedParams<df64>&, BatchMask,
                                                 cudaStream_t);
template bool ct_axis0_stiffness_staged<df64, 3>(int, cplx<df64>*, int64_t, int64_t, int64_t,
                                                 int, const FusedParams<df64>&, BatchMask,
                                                 cudaStream_t);

bool ct_axis0_stiffness_tma_df(int n0, cplx<df64>* X, int64_t P, int64_t cstride,
                               int64_t bstride, int batch, const FusedParams<df64>& fp,
                               BatchMask mask, cudaStream_t st) {
  return ct_axis0_stiffness_tma<df64, false>(n0, false, X, P, cstride, bstride, batch, fp,
                                             mask, st);
}

void ct_set_smem_attrs_df_axis0(size_t max_smem) {
#define CASE(N)                                                                          \
  if constexpr (ct_has<df64>(N)) {                                                       \
    cudaFuncSetAttribute(axis0_stiffness_staged<df64, 2, CtEng<N, 8>>,                   \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(axis0_stiffness_staged<df64, 3, CtEng<N, 8>>,                   \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
  }
  BRI17_CT_CASES(CASE)
#undef CASE
  ct_set_smem_attrs_tma<df64, false>(max_smem);
}

cudaError_t tma_set_wait_limit_df(uint64_t ns) {
  const unsigned long long v = ns;
  return cudaMemcpyToSymbol(g_tma_wait_limit_ns, &v, sizeof(v));
}

cudaError_t tma_wait_timeouts_df(int* count) {
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
