// Compile-time-length power-of-two passes, FP32 instances, and the
// TMA-staged axis-0 stiffness pass (FP32 only: at FP64 the pass is bound by
// the FP64 pipe, not by memory).
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT_INSTANTIATE(float)

namespace {

// Lines per CTA: 128-byte rows of the tile (16 complex64) up to n0 = 128,
// 64-byte rows at 256, 32-byte rows from 512 (a 68 KB tile, three CTAs per
// SM); at most 256 threads.
constexpr int tma_lines(int n0) { return n0 <= 128 ? 16 : n0 <= 256 ? 8 : n0 <= 512 ? 4 : 2; }

template <int N>
int tma_pitch() {
  return exchange_pitch(N, tma_lines(N), (int)sizeof(cplx<float>), true);
}

template <int N>
size_t tma_smem_bytes() {
  constexpr int TB = tma_lines(N);
  return ((size_t)3 * N * TB + (size_t)TB * tma_pitch<N>() + N) * sizeof(cplx<float>) + 16;
}

}  // namespace

bool ct_axis0_stiffness_tma_f32(int n0, bool keep, cplx<float>* X, int64_t P, int64_t cstride,
                                int64_t bstride, int batch, const FusedParams<float>& fp,
                                BatchMask mask, cudaStream_t st) {
  constexpr int DIM = 3;
  // The map's strides (P and cstride complex64) must be multiples of 16
  // bytes, the base 16-byte aligned, and the planes evenly spaced.
  if (P % 2 != 0 || cstride != (int64_t)n0 * P || bstride != DIM * cstride) return false;
  if (reinterpret_cast<uintptr_t>(X) % 16 != 0) return false;
  if ((int64_t)P * 2 >= ((int64_t)1 << 31)) return false;
  switch (n0) {
#define CASE(N)                                                                         \
  case N: {                                                                             \
    constexpr int E = 8;                                                                \
    constexpr int TT = N / E;                                                           \
    constexpr int TB = tma_lines(N);                                                    \
    static_assert(TT * TB <= 256 && TB % 2 == 0, "tile shape");                         \
    const int rows = N < 256 ? N : 256;                                                 \
    CUtensorMap map;                                                                    \
    if (!encode_tiled_map_3d(&map, X, (int)sizeof(float), (uint64_t)P * 2, N,           \
                             (uint64_t)DIM * batch, (uint64_t)P * sizeof(cplx<float>),  \
                             (uint64_t)cstride * sizeof(cplx<float>), 2 * TB, rows))    \
      return false;                                                                     \
    dim3 grid((unsigned)((P + TB - 1) / TB), (unsigned)batch);                          \
    if (keep)                                                                           \
      launch_pdl(axis0_stiffness_tma<float, DIM, CtEng<N, E>, true>, grid, TT * TB,     \
                 tma_smem_bytes<N>(), st, map, P, TB, tma_pitch<N>(), CtEng<N, E>{}, fp, \
                 mask);                                                                 \
    else                                                                                \
      launch_pdl(axis0_stiffness_tma<float, DIM, CtEng<N, E>, false>, grid, TT * TB,    \
                 tma_smem_bytes<N>(), st, map, P, TB, tma_pitch<N>(), CtEng<N, E>{}, fp, \
                 mask);                                                                 \
    return true;                                                                        \
  }
    CASE(16) CASE(32) CASE(64) CASE(128) CASE(256) CASE(512) CASE(1024)
#undef CASE
    default:
      return false;
  }
}

void ct_set_smem_attrs_tma_f32(size_t max_smem) {
#define CASE(N)                                                                          \
  cudaFuncSetAttribute(axis0_stiffness_tma<float, 3, CtEng<N, 8>, false>,                \
                       cudaFuncAttributeMaxDynamicSharedMemorySize,                      \
                       (int)std::min(max_smem, tma_smem_bytes<N>()));                    \
  cudaFuncSetAttribute(axis0_stiffness_tma<float, 3, CtEng<N, 8>, true>,                 \
                       cudaFuncAttributeMaxDynamicSharedMemorySize,                      \
                       (int)std::min(max_smem, tma_smem_bytes<N>()));
  CASE(16) CASE(32) CASE(64) CASE(128) CASE(256) CASE(512) CASE(1024)
#undef CASE
  cudaGetLastError();
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
