// passes_ct.cuh -- launchers of the compile-time-length instances of the
// power-of-two passes; passes_ct_f32.cu and passes_ct_f64.cu instantiate
// them for one scalar type each (separate translation units build in
// parallel).
#pragma once

#include "passes_p2.cuh"

namespace bri17gb {

#define BRI17_CT_CASES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)

template <typename T>
bool ct_rows_r2c(int m, const T* x, cplx<T>* X, int64_t nrows, int H, const cplx<T>* tw,
                 int RB, size_t smem, BatchMask mask, cudaStream_t st) {
  const unsigned grid = (unsigned)((nrows + RB - 1) / RB);
  switch (m) {
#define CASE(N)                                                                      \
  case N:                                                                            \
    if (N > 512) return false;                                                       \
    rows_r2c_p2<T, CtEng<N>><<<grid, (N / 8) * RB, smem, st>>>(x, X, nrows, H,       \
                                                               CtEng<N>{}, tw, RB, mask); \
    return true;
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T>
bool ct_rows_c2r(int m, const cplx<T>* X, T* x, int64_t nrows, int H, const cplx<T>* tw,
                 int RB, size_t smem, BatchMask mask, cudaStream_t st) {
  const unsigned grid = (unsigned)((nrows + RB - 1) / RB);
  switch (m) {
#define CASE(N)                                                                      \
  case N:                                                                            \
    if (N > 512) return false;                                                       \
    rows_c2r_p2<T, CtEng<N>><<<grid, (N / 8) * RB, smem, st>>>(X, x, nrows, H,       \
                                                               CtEng<N>{}, tw, RB, mask); \
    return true;
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T, bool INV>
bool ct_axis_c2c(int n, cplx<T>* X, int64_t B, int TB, dim3 grid, size_t smem,
                 const cplx<T>* tw, BatchMask mask, cudaStream_t st) {
  switch (n) {
#define CASE(N)                                                                       \
  case N:                                                                             \
    axis_c2c_p2<T, INV, CtEng<N>><<<grid, (N / 8) * TB, smem, st>>>(X, B, TB, CtEng<N>{}, \
                                                                    tw, mask);        \
    return true;
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T, int DIM>
bool ct_axis0_stiffness(int n0, cplx<T>* X, int64_t P, int64_t cstride, int64_t bstride,
                        int TB, dim3 grid, size_t smem, const FusedParams<T>& fp,
                        BatchMask mask, cudaStream_t st) {
  switch (n0) {
#define CASE(N)                                                                  \
  case N:                                                                        \
    axis0_stiffness_p2<T, DIM, CtEng<N>><<<grid, (N / 8) * TB, smem, st>>>(     \
        X, P, cstride, bstride, TB, CtEng<N>{}, fp, mask);                      \
    return true;
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T>
void ct_set_smem_attrs_t(size_t max_smem) {
#define CASE(N)                                                                              \
  cudaFuncSetAttribute(rows_r2c_p2<T, CtEng<N>>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                       (int)max_smem);                                                       \
  cudaFuncSetAttribute(rows_c2r_p2<T, CtEng<N>>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                       (int)max_smem);                                                       \
  cudaFuncSetAttribute(axis_c2c_p2<T, false, CtEng<N>>,                                      \
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);          \
  cudaFuncSetAttribute(axis_c2c_p2<T, true, CtEng<N>>,                                       \
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);          \
  cudaFuncSetAttribute(axis0_stiffness_p2<T, 2, CtEng<N>>,                                   \
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);          \
  cudaFuncSetAttribute(axis0_stiffness_p2<T, 3, CtEng<N>>,                                   \
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  BRI17_CT_CASES(CASE)
#undef CASE
  cudaGetLastError();
}

#define BRI17_CT_INSTANTIATE(T)                                                             \
  template bool ct_rows_r2c<T>(int, const T*, cplx<T>*, int64_t, int, const cplx<T>*, int, \
                               size_t, BatchMask, cudaStream_t);                           \
  template bool ct_rows_c2r<T>(int, const cplx<T>*, T*, int64_t, int, const cplx<T>*, int, \
                               size_t, BatchMask, cudaStream_t);                           \
  template bool ct_axis_c2c<T, false>(int, cplx<T>*, int64_t, int, dim3, size_t,            \
                                      const cplx<T>*, BatchMask, cudaStream_t);             \
  template bool ct_axis_c2c<T, true>(int, cplx<T>*, int64_t, int, dim3, size_t,             \
                                     const cplx<T>*, BatchMask, cudaStream_t);              \
  template bool ct_axis0_stiffness<T, 2>(int, cplx<T>*, int64_t, int64_t, int64_t, int,     \
                                         dim3, size_t, const FusedParams<T>&, BatchMask,    \
                                         cudaStream_t);                                     \
  template bool ct_axis0_stiffness<T, 3>(int, cplx<T>*, int64_t, int64_t, int64_t, int,     \
                                         dim3, size_t, const FusedParams<T>&, BatchMask,    \
                                         cudaStream_t);                                     \
  template void ct_set_smem_attrs_t<T>(size_t);

}  // namespace bri17gb
