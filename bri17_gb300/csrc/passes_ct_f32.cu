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

// Raises a kernel's dynamic shared-memory limit to what the SM allows next
// to its static shared memory (kernels with a block reduction declare some:
// asking for the full max_smem would be refused and leave the 48 KB default).
template <typename K>
static void set_dyn_smem(K kernel, size_t max_smem) {
  cudaFuncAttributes a;
  if (cudaFuncGetAttributes(&a, kernel) != cudaSuccess) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(max_smem - a.sharedSizeBytes));
}

void ct_set_smem_attrs_tma_f32(size_t max_smem) {
  ct_set_smem_attrs_tma<float>(max_smem);
#define CASE(N)                                                                          \
  if constexpr (N >= 16)                                                                 \
    set_dyn_smem(axis0_stiffness_tma<float, 3, CtEng<N, 8>, false, true>, max_smem);     \
  set_dyn_smem(axis0_stiffness_staged<float, 3, CtEng<N, 8>, true>, max_smem);           \
  if constexpr (N <= 512) {                                                              \
    set_dyn_smem(rows_r2c_cg<CtEng<N, 8>>, max_smem);                                    \
    set_dyn_smem(rows_c2r_cg<CtEng<N, 8>>, max_smem);                                    \
  }
  BRI17_CT_CASES(CASE)
#undef CASE
  cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The fused CG iteration's passes (FP32, 3D, compile-time lengths).

int ct_rows_ctas(int m, int64_t nrows, const BatchMask& mask) {
  if (m < 8 || m > 512 || (m & (m - 1))) return 0;
  const int rb = ct_rows_per_cta(m / 8, nrows, mask);
  return (int)((nrows + rb - 1) / rb);
}

bool ct_rows_r2c_cg(int m, CgRows<float> cg, cplx<float>* X, int64_t nrows, int H,
                    const cplx<float>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                        \
  case N: {                                                                           \
    if constexpr (N > 512) {                                                          \
      return false;                                                                   \
    } else {                                                                          \
      const int TT = N / 8;                                                           \
      const int rb = ct_rows_per_cta(TT, nrows, mask);                                \
      const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<float>), false);       \
      const size_t smem = (3 * N + 1 + (size_t)rb * pitch) * sizeof(cplx<float>);     \
      launch_pdl(rows_r2c_cg<CtEng<N, 8>>, (unsigned)((nrows + rb - 1) / rb), TT * rb, \
                 smem, st, cg, X, nrows, H, CtEng<N, 8>{}, tw, rb, pitch, mask);      \
      return true;                                                                    \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool ct_rows_c2r_cg(int m, const cplx<float>* X, CgRows<float> cg, int64_t nrows, int H,
                    const cplx<float>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                        \
  case N: {                                                                           \
    if constexpr (N > 512) {                                                          \
      return false;                                                                   \
    } else {                                                                          \
      const int TT = N / 8;                                                           \
      const int rb = ct_rows_per_cta(TT, nrows, mask);                                \
      const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<float>), false);       \
      const size_t smem = (3 * N + (size_t)rb * pitch) * sizeof(cplx<float>);         \
      launch_pdl(rows_c2r_cg<CtEng<N, 8>>, (unsigned)((nrows + rb - 1) / rb), TT * rb, \
                 smem, st, X, cg, nrows, H, CtEng<N, 8>{}, tw, rb, pitch, mask);      \
      return true;                                                                    \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool ct_axis0_cg_dot_f32(int n0, int form, cplx<float>* X, int64_t P, int64_t cstride,
                         const FusedParams<float>& fp, BatchMask mask, cudaStream_t st,
                         int64_t* nctas) {
  constexpr int DIM = 3;
  const bool tma_ok = (form == 2 || form == 3) &&
                      (P * (int64_t)sizeof(cplx<float>)) % 16 == 0 &&
                      cstride == (int64_t)n0 * P && reinterpret_cast<uintptr_t>(X) % 16 == 0 &&
                      (int64_t)P * 2 < ((int64_t)1 << 31);
  switch (n0) {
#define CASE(N)                                                                          \
  case N: {                                                                             \
    if constexpr (N >= 16) {                                                            \
      if (tma_ok) {                                                                     \
        constexpr int TB = tma_lines<float>(N);                                         \
        const int rows = N < 256 ? N : 256;                                             \
        CUtensorMap map;                                                                \
        if (encode_tiled_map_3d(&map, X, (int)sizeof(float), (uint64_t)P * 2, N,        \
                                (uint64_t)DIM, (uint64_t)P * sizeof(cplx<float>),        \
                                (uint64_t)cstride * sizeof(cplx<float>), 2 * TB, rows)) { \
          dim3 grid((unsigned)((P + TB - 1) / TB), 1u);                                 \
          launch_pdl(axis0_stiffness_tma<float, DIM, CtEng<N, 8>, false, true>, grid,    \
                     (N / 8) * TB, tma_smem_bytes<float, N>(), st, map, P, TB,           \
                     tma_pitch<float, N>(), CtEng<N, 8>{}, fp, mask);                    \
          *nctas = grid.x;                                                              \
          return true;                                                                  \
        }                                                                               \
      }                                                                                 \
    }                                                                                   \
    const int TT = N / 8;                                                               \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, P));    \
    const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<float>), true);            \
    const size_t smem = (N + (size_t)TB * pitch +                                       \
                         (size_t)DIM * TB * stash_pitch(N, TB, sizeof(cplx<float>))) *  \
                        sizeof(cplx<float>);                                            \
    dim3 grid((unsigned)((P + TB - 1) / TB), 1u);                                       \
    launch_pdl(axis0_stiffness_staged<float, DIM, CtEng<N, 8>, true>, grid, TT * TB, smem, \
               st, X, P, cstride, (int64_t)DIM * cstride, TB, pitch, CtEng<N, 8>{}, fp,  \
               mask);                                                                   \
    *nctas = grid.x;                                                                    \
    return true;                                                                        \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

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
