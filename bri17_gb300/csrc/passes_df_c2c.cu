// Float-pair (df64.cuh) instances of the axis-1 passes.
#include "passes_ct.cuh"

namespace bri17gb {

template bool ct_axis_c2c<df64, false>(int, cplx<df64>*, int64_t, int64_t, const cplx<df64>*,
                                       BatchMask, cudaStream_t);
template bool ct_axis_c2c<df64, true>(int, cplx<df64>*, int64_t, int64_t, const cplx<df64>*,
                                      BatchMask, cudaStream_t);

void ct_set_smem_attrs_df_c2c(size_t max_smem) {
#define CASE(N)                                                                          \
  if constexpr (ct_has<df64>(N)) {                                                       \
    cudaFuncSetAttribute(axis_c2c_p2<df64, false, CtEng<N, 8>>,                          \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(axis_c2c_p2<df64, true, CtEng<N, 8>>,                           \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
  }
  BRI17_CT_CASES(CASE)
#undef CASE
}

}  // namespace bri17gb
