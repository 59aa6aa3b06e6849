// Float-pair (df64.cuh) instances of the last-axis passes: FP64 fields in
// memory, converted to and from float pairs at load and store.
#include "passes_ct.cuh"

namespace bri17gb {

template bool ct_rows_r2c<df64>(int, const double*, cplx<df64>*, int64_t, int,
                                const cplx<df64>*, BatchMask, cudaStream_t);
template bool ct_rows_c2r<df64>(int, const cplx<df64>*, double*, int64_t, int,
                                const cplx<df64>*, BatchMask, cudaStream_t);

void ct_set_smem_attrs_df_rows(size_t max_smem) {
#define CASE(N)                                                                          \
  if constexpr (ct_has<df64>(N) && N <= 512) {                                           \
    cudaFuncSetAttribute(rows_r2c_p2<df64, CtEng<N, 8>>,                                 \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(rows_c2r_p2<df64, CtEng<N, 8>>,                                 \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
  }
  BRI17_CT_CASES(CASE)
#undef CASE
}

}  // namespace bri17gb
