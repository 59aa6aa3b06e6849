// passes_ct.cuh -- launchers of the compile-time-length instances of the
// power-of-two passes; passes_ct_f32.cu and passes_ct_f64.cu instantiate
// them for one scalar type each (separate translation units build in
// parallel).  Every launch carries the programmatic-dependent-launch
// attribute (see pdl.cuh).
#pragma once

#include <algorithm>
#include <cstring>
#include <cstdlib>
#include <type_traits>

#include "passes_p2.cuh"

namespace bri17gb {

#define BRI17_CT_CASES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)

// Lengths with compile-time instances per scalar type: every case of
// BRI17_CT_CASES for FP32 and FP64; 64..512 for float pairs (their kernels
// are long to compile, and the grids that use them are 64..1024 per axis).
template <typename T>
constexpr bool ct_has(int n) {
  return std::is_same<T, df64>::value ? (n >= 64 && n <= 512) : true;
}

// Elements per thread for scalar T and line length N (single-component
// passes); the fused axis-0 pass holds DIM components per thread and uses 8.
template <typename T, int N>
struct CtE {
  // 16 elements per thread was measured slower than 8 for the FP32 row
  // passes (fewer threads per row, longer dependency chains): 8 throughout.
  static constexpr int value = 8;
};
constexpr int kFusedE = 8;

// Rows per CTA for the last-axis passes: kP2Threads threads' worth, a power
// of two dividing the rows of one batch entry when masked.
inline int ct_rows_per_cta(int T, int64_t nrows, const BatchMask& mask) {
  int rb = std::max(1, kP2Threads / T);
  if (mask.flags)
    while (rb > 1 && mask.unit % rb != 0) rb /= 2;
  return (int)std::max<int64_t>(1, std::min<int64_t>(rb, nrows));
}

template <typename T>
bool ct_rows_r2c(int m, const typename IoOf<T>::type* x, cplx<T>* X, int64_t nrows, int H,
                 const cplx<T>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                       \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    if (N > 512) return false;                                                        \
    constexpr int E = CtE<T, N>::value;                                               \
    const int TT = N / E;                                                             \
    const int rb = ct_rows_per_cta(TT, nrows, mask);                                  \
    const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<T>), false);             \
    const size_t smem = (3 * N + 1 + (size_t)rb * pitch) * sizeof(cplx<T>);           \
    launch_pdl(rows_r2c_p2<T, CtEng<N, E>>, (unsigned)((nrows + rb - 1) / rb), TT * rb, smem, st,  \
        x, X, nrows, H, CtEng<N, E>{}, tw, rb, pitch, mask);                          \
    return true;                                                                      \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T>
bool ct_rows_c2r(int m, const cplx<T>* X, typename IoOf<T>::type* x, int64_t nrows, int H,
                 const cplx<T>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                       \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    if (N > 512) return false;                                                        \
    constexpr int E = CtE<T, N>::value;                                               \
    const int TT = N / E;                                                             \
    const int rb = ct_rows_per_cta(TT, nrows, mask);                                  \
    const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<T>), false);             \
    const size_t smem = (3 * N + (size_t)rb * pitch) * sizeof(cplx<T>);               \
    launch_pdl(rows_c2r_p2<T, CtEng<N, E>>, (unsigned)((nrows + rb - 1) / rb), TT * rb, smem, st,  \
        X, x, nrows, H, CtEng<N, E>{}, tw, rb, pitch, mask);                          \
    return true;                                                                      \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

// Sixteen elements per thread in the FP32 axis-1 pass for lengths 256 and
// 512: one shared-memory exchange fewer per transform and 16 (256) or 8
// (512) lines per CTA; 4-5% faster there, 2% slower at 128, which keeps
// eight (BRI17_C2C_E=8 keeps eight everywhere, for measurements).
inline bool c2c_e16() {
  static const bool on = [] {
    const char* e = getenv("BRI17_C2C_E");
    return !(e && strcmp(e, "8") == 0);
  }();
  return on;
}

template <typename T, bool INV>
bool ct_axis_c2c(int n, cplx<T>* X, int64_t B, int64_t nouter, const cplx<T>* tw,
                 BatchMask mask, cudaStream_t st) {
  switch (n) {
#define CASE(N)                                                                        \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    if constexpr (std::is_same<T, float>::value && N >= 256 && N <= 512) {             \
      if (c2c_e16()) {                                                                 \
        constexpr int E16 = 16;                                                        \
        const int TT = N / E16;                                                        \
        const int TB =                                                                 \
            (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, nouter * B)); \
        const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<T>), true, E16);      \
        const size_t smem = (N + (size_t)TB * pitch) * sizeof(cplx<T>);                \
        const int64_t nl = nouter * B;                                                 \
        launch_pdl(axis_c2c_p2<T, INV, CtEng<N, E16>>, (unsigned)((nl + TB - 1) / TB),  \
                   TT * TB, smem, st, X, B, nl, TB, CtEng<N, E16>{}, tw, pitch, mask); \
        return true;                                                                   \
      }                                                                                \
    }                                                                                  \
    constexpr int E = CtE<T, N>::value;                                                \
    const int TT = N / E;                                                              \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, nouter * B)); \
    const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<T>), true);               \
    const size_t smem = (N + (size_t)TB * pitch) * sizeof(cplx<T>);                    \
    const int64_t nl = nouter * B;                                                     \
    launch_pdl(axis_c2c_p2<T, INV, CtEng<N, E>>, (unsigned)((nl + TB - 1) / TB), TT * TB, \
               smem, st, X, B, nl, TB, CtEng<N, E>{}, tw, pitch, mask);                \
    return true;                                                                       \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T, int DIM>
bool ct_axis0_stiffness(int n0, cplx<T>* X, int64_t P, int64_t cstride, int64_t bstride,
                        int batch, const FusedParams<T>& fp, BatchMask mask,
                        cudaStream_t st) {
  switch (n0) {
#define CASE(N)                                                                        \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    constexpr int E = kFusedE;                                                         \
    const int TT = N / E;                                                              \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2FusedThreads / TT, P)); \
    const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<T>), true);               \
    const size_t smem = (N + (size_t)TB * pitch) * sizeof(cplx<T>);                    \
    dim3 grid((unsigned)((P + TB - 1) / TB), (unsigned)batch);                         \
    launch_pdl(axis0_stiffness_p2<T, DIM, CtEng<N, E>>, grid, TT * TB, smem, st,               \
        X, P, cstride, bstride, TB, pitch, CtEng<N, E>{}, fp, mask);                   \
    return true;                                                                       \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

// Staged form: TB lines per CTA with kP2Threads threads (at least 8
// consecutive lines for 64-byte segments), 1 + 1 + DIM lines of shared
// memory per line of the tile.
template <typename T, int DIM>
bool ct_axis0_stiffness_staged(int n0, cplx<T>* X, int64_t P, int64_t cstride,
                               int64_t bstride, int batch, const FusedParams<T>& fp,
                               BatchMask mask, cudaStream_t st) {
  switch (n0) {
#define CASE(N)                                                                        \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    constexpr int E = 8;                                                               \
    const int TT = N / E;                                                              \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, P));   \
    const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<T>), true);               \
    const size_t smem = (N + (size_t)TB * pitch + (size_t)DIM * TB * stash_pitch(N, TB, sizeof(cplx<T>))) * sizeof(cplx<T>);     \
    dim3 grid((unsigned)((P + TB - 1) / TB), (unsigned)batch);                         \
    launch_pdl(axis0_stiffness_staged<T, DIM, CtEng<N, E>>, grid, TT * TB, smem, st,   \
               X, P, cstride, bstride, TB, pitch, CtEng<N, E>{}, fp, mask);            \
    return true;                                                                       \
    }                                                                                 \
  }
    BRI17_CT_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

// TMA-staged form (3D): lines per CTA give tile rows of 128 bytes up to
// n0 = 128, 64 bytes at 256 and 32 bytes from 512, with at most 256 threads
// and at least two lines (the copies' x offsets stay 16-byte multiples).
template <typename T>
constexpr int tma_lines(int n0) {
  const int bytes = n0 <= 128 ? 128 : n0 <= 256 ? 64 : 32;
  const int cap = 256 / (n0 / 8 > 0 ? n0 / 8 : 1);
  const int tb = bytes / (int)sizeof(cplx<T>) < cap ? bytes / (int)sizeof(cplx<T>) : cap;
  return tb < 2 ? 2 : tb;
}

template <typename T, int N>
int tma_pitch() {
  return exchange_pitch(N, tma_lines<T>(N), (int)sizeof(cplx<T>), true);
}

// Float pairs exchange inside the tile (axis0_stiffness_tma's XS) when a
// tile row is 128 bytes, TB = 8 lines of 16 bytes (n0 = 64, 128): 0
// otherwise, and for FP32, whose staged compute keeps its exchange buffer.
template <typename T, int N>
constexpr int tma_xs() {
  return std::is_same<T, df64>::value && tma_lines<T>(N) * (int)sizeof(cplx<T>) == 128
             ? tma_lines<T>(N)
             : 0;
}

// Shared memory the p.Kp reduction of the PQ instance adds after the
// mbarrier: 8 warp sums and the last-CTA flag.
constexpr size_t kTmaPqSmem = 80;

// Dynamic shared memory of the staged-compute instance (XS = tma_xs) or,
// with xs = 0 forced, of the instances with an exchange buffer.
template <typename T, int N>
size_t tma_smem_bytes(bool with_exchange = tma_xs<T, N>() == 0) {
  constexpr int TB = tma_lines<T>(N);
  const size_t exch = with_exchange ? (size_t)TB * tma_pitch<T, N>() : 0;
  return ((size_t)3 * N * TB + exch + N) * sizeof(cplx<T>) + 16;
}

// WITH_KEEP = false compiles only the staged-compute variant (keep is then
// ignored).
template <typename T, bool WITH_KEEP = true>
bool ct_axis0_stiffness_tma(int n0, bool keep, cplx<T>* X, int64_t P, int64_t cstride,
                            int64_t bstride, int batch, const FusedParams<T>& fp,
                            BatchMask mask, cudaStream_t st) {
  constexpr int DIM = 3;
  constexpr int kPer = (int)(sizeof(cplx<T>) / sizeof(T));
  // The map's strides (P and cstride complex) must be multiples of 16
  // bytes, the base 16-byte aligned, and the planes evenly spaced.
  if (!tma_layout_ok<T>(X, P, cstride, bstride, n0)) return false;
  switch (n0) {
#define CASE(N)                                                                          \
  case N: {                                                                           \
    if constexpr (!ct_has<T>(N)) {                                                    \
      return false;                                                                   \
    } else {                                                                          \
    constexpr int E = 8;                                                                 \
    constexpr int TT = N / E;                                                            \
    constexpr int TB = tma_lines<T>(N);                                                  \
    static_assert(TT * TB <= 256 && TB % 2 == 0, "tile shape");                          \
    const int rows = N < 256 ? N : 256;                                                  \
    CUtensorMap map;                                                                     \
    if (!encode_tiled_map_3d(&map, X, (int)sizeof(T), (uint64_t)P * kPer, N,             \
                             (uint64_t)DIM * batch, (uint64_t)P * sizeof(cplx<T>),       \
                             (uint64_t)cstride * sizeof(cplx<T>), kPer * TB, rows))      \
      return false;                                                                      \
    dim3 grid((unsigned)((P + TB - 1) / TB), (unsigned)batch);                           \
    bool launched = false;                                                               \
    if constexpr (WITH_KEEP) {                                                           \
      if (keep) {                                                                        \
        launch_pdl(axis0_stiffness_tma<T, DIM, CtEng<N, E>, true>, grid, TT * TB,        \
                   tma_smem_bytes<T, N>(true), st, map, P, TB, tma_pitch<T, N>(),        \
                   CtEng<N, E>{}, fp, mask);                                             \
        launched = true;                                                                 \
      }                                                                                  \
    }                                                                                    \
    if constexpr (std::is_same<T, float>::value) {                                       \
      if (!launched && fp.cg) {                                                          \
        if (batch != 1) return false;                                                    \
        launch_pdl(axis0_stiffness_tma<T, DIM, CtEng<N, E>, false, true>, grid, TT * TB, \
                   tma_smem_bytes<T, N>(true) + kTmaPqSmem, st, map, P, TB,              \
                   tma_pitch<T, N>(), CtEng<N, E>{}, fp, mask);                          \
        launched = true;                                                                 \
      }                                                                                  \
    }                                                                                    \
    if (!launched)                                                                       \
      launch_pdl(axis0_stiffness_tma<T, DIM, CtEng<N, E>, false, false, tma_xs<T, N>()>, \
                 grid, TT * TB, tma_smem_bytes<T, N>(), st, map, P, TB, tma_pitch<T, N>(), \
                 CtEng<N, E>{}, fp, mask);                                               \
    return true;                                                                         \
    }                                                                                 \
  }
    CASE(16) CASE(32) CASE(64) CASE(128) CASE(256) CASE(512) CASE(1024)
#undef CASE
    default:
      return false;
  }
}

template <typename T, bool WITH_KEEP = true>
void ct_set_smem_attrs_tma(size_t max_smem) {
#define CASE(N)                                                                          \
  if constexpr (ct_has<T>(N)) {                                                          \
    cudaFuncSetAttribute(axis0_stiffness_tma<T, 3, CtEng<N, 8>, false, false, tma_xs<T, N>()>, \
                         cudaFuncAttributeMaxDynamicSharedMemorySize,                    \
                         (int)std::min(max_smem, tma_smem_bytes<T, N>()));               \
    if constexpr (WITH_KEEP)                                                             \
      cudaFuncSetAttribute(axis0_stiffness_tma<T, 3, CtEng<N, 8>, true>,                 \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,                  \
                           (int)std::min(max_smem, tma_smem_bytes<T, N>(true)));         \
    if constexpr (std::is_same<T, float>::value)                                         \
      cudaFuncSetAttribute(axis0_stiffness_tma<T, 3, CtEng<N, 8>, false, true>,          \
                           cudaFuncAttributeMaxDynamicSharedMemorySize,                  \
                           (int)std::min(max_smem, tma_smem_bytes<T, N>(true) + kTmaPqSmem)); \
  }
  CASE(16) CASE(32) CASE(64) CASE(128) CASE(256) CASE(512) CASE(1024)
#undef CASE
  cudaGetLastError();
}

template <typename T>
void ct_set_smem_attrs_t(size_t max_smem) {
  if constexpr (std::is_same<T, float>::value) {
#define CASE16(N)                                                                      \
    cudaFuncSetAttribute(axis_c2c_p2<T, false, CtEng<N, 16>>,                          \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis_c2c_p2<T, true, CtEng<N, 16>>,                           \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
    CASE16(256) CASE16(512)
#undef CASE16
  }
#define CASE(N)                                                                        \
  {                                                                                    \
    constexpr int E = CtE<T, N>::value;                                                \
    cudaFuncSetAttribute(rows_r2c_p2<T, CtEng<N, E>>,                                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(rows_c2r_p2<T, CtEng<N, E>>,                                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis_c2c_p2<T, false, CtEng<N, E>>,                           \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis_c2c_p2<T, true, CtEng<N, E>>,                            \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis0_stiffness_p2<T, 2, CtEng<N, kFusedE>>,                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis0_stiffness_p2<T, 3, CtEng<N, kFusedE>>,                  \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis0_stiffness_staged<T, 2, CtEng<N, 8>>,                    \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
    cudaFuncSetAttribute(axis0_stiffness_staged<T, 3, CtEng<N, 8>>,                    \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);  \
  }
  BRI17_CT_CASES(CASE)
#undef CASE
  cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Lengths 3 * 2^k on the twelve-element engine (CtEng3), FP32 and FP64:
// 24..192 per strided axis, 48..384 on the last axis (rows of 24..192
// complex points).  Same kernels and block shapes as the power-of-two
// instances; the axis-0 pass takes the staged form (the registers form
// holds 3 x 12 complex values per thread: 255 registers with spills in
// FP32, against 84-118 staged).
#define BRI17_CT3_CASES(X) X(24) X(48) X(96) X(192)

template <typename T>
bool ct3_rows_r2c(int m, const typename IoOf<T>::type* x, cplx<T>* X, int64_t nrows, int H,
                  const cplx<T>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                         \
  case N: {                                                                             \
    using Eng = CtEng3<N>;                                                              \
    const int TT = Eng::kTT;                                                            \
    const int rb = ct_rows_per_cta(TT, nrows, mask);                                    \
    const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<T>), false, Eng::E);       \
    const size_t smem = (3 * N + 1 + (size_t)rb * pitch) * sizeof(cplx<T>);             \
    launch_pdl(rows_r2c_p2<T, Eng>, (unsigned)((nrows + rb - 1) / rb), TT * rb, smem, st, \
               x, X, nrows, H, Eng{}, tw, rb, pitch, mask);                             \
    return true;                                                                        \
  }
    BRI17_CT3_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T>
bool ct3_rows_c2r(int m, const cplx<T>* X, typename IoOf<T>::type* x, int64_t nrows, int H,
                  const cplx<T>* tw, BatchMask mask, cudaStream_t st) {
  switch (m) {
#define CASE(N)                                                                         \
  case N: {                                                                             \
    using Eng = CtEng3<N>;                                                              \
    const int TT = Eng::kTT;                                                            \
    const int rb = ct_rows_per_cta(TT, nrows, mask);                                    \
    const int pitch = exchange_pitch(N, rb, (int)sizeof(cplx<T>), false, Eng::E);       \
    const size_t smem = (3 * N + (size_t)rb * pitch) * sizeof(cplx<T>);                 \
    launch_pdl(rows_c2r_p2<T, Eng>, (unsigned)((nrows + rb - 1) / rb), TT * rb, smem, st, \
               X, x, nrows, H, Eng{}, tw, rb, pitch, mask);                             \
    return true;                                                                        \
  }
    BRI17_CT3_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T, bool INV>
bool ct3_axis_c2c(int n, cplx<T>* X, int64_t B, int64_t nouter, const cplx<T>* tw,
                  BatchMask mask, cudaStream_t st) {
  switch (n) {
#define CASE(N)                                                                          \
  case N: {                                                                              \
    using Eng = CtEng3<N>;                                                               \
    const int TT = Eng::kTT;                                                             \
    const int64_t nl = nouter * B;                                                       \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, nl));    \
    const int pitch = exchange_pitch(N, TB, (int)sizeof(cplx<T>), true, Eng::E);         \
    const size_t smem = (N + (size_t)TB * pitch) * sizeof(cplx<T>);                      \
    launch_pdl(axis_c2c_p2<T, INV, Eng>, (unsigned)((nl + TB - 1) / TB), TT * TB, smem, st, \
               X, B, nl, TB, Eng{}, tw, pitch, mask);                                    \
    return true;                                                                         \
  }
    BRI17_CT3_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T, int DIM>
bool ct3_axis0_stiffness(int n0, cplx<T>* X, int64_t P, int64_t cstride, int64_t bstride,
                         int batch, const FusedParams<T>& fp, BatchMask mask, cudaStream_t st) {
  constexpr size_t csz = sizeof(cplx<T>);
  switch (n0) {
#define CASE(N)                                                                          \
  case N: {                                                                              \
    using Eng = CtEng3<N>;                                                               \
    const int TT = Eng::kTT;                                                             \
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2Threads / TT, P));     \
    const int pitch = exchange_pitch(N, TB, (int)csz, true, Eng::E);                     \
    const size_t smem =                                                                  \
        (N + (size_t)TB * pitch + (size_t)DIM * TB * stash_pitch(N, TB, (int)csz)) * csz; \
    dim3 grid((unsigned)((P + TB - 1) / TB), (unsigned)batch);                           \
    launch_pdl(axis0_stiffness_staged<T, DIM, Eng>, grid, TT * TB, smem, st, X, P, cstride, \
               bstride, TB, pitch, Eng{}, fp, mask);                                     \
    return true;                                                                         \
  }
    BRI17_CT3_CASES(CASE)
#undef CASE
    default:
      return false;
  }
}

template <typename T>
void ct3_set_smem_attrs_t(size_t max_smem) {
#define CASE(N)                                                                          \
  {                                                                                      \
    using Eng = CtEng3<N>;                                                               \
    cudaFuncSetAttribute(rows_r2c_p2<T, Eng>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                         (int)max_smem);                                                 \
    cudaFuncSetAttribute(rows_c2r_p2<T, Eng>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                         (int)max_smem);                                                 \
    cudaFuncSetAttribute(axis_c2c_p2<T, false, Eng>,                                     \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(axis_c2c_p2<T, true, Eng>,                                      \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(axis0_stiffness_staged<T, 2, Eng>,                              \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
    cudaFuncSetAttribute(axis0_stiffness_staged<T, 3, Eng>,                              \
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);    \
  }
  BRI17_CT3_CASES(CASE)
#undef CASE
  cudaGetLastError();
}

#define BRI17_CT3_INSTANTIATE(T)                                                             \
  template bool ct3_rows_r2c<T>(int, const typename IoOf<T>::type*, cplx<T>*, int64_t, int, \
                                const cplx<T>*, BatchMask, cudaStream_t);                   \
  template bool ct3_rows_c2r<T>(int, const cplx<T>*, typename IoOf<T>::type*, int64_t, int, \
                                const cplx<T>*, BatchMask, cudaStream_t);                   \
  template bool ct3_axis_c2c<T, false>(int, cplx<T>*, int64_t, int64_t, const cplx<T>*,      \
                                       BatchMask, cudaStream_t);                             \
  template bool ct3_axis_c2c<T, true>(int, cplx<T>*, int64_t, int64_t, const cplx<T>*,       \
                                      BatchMask, cudaStream_t);                              \
  template bool ct3_axis0_stiffness<T, 2>(int, cplx<T>*, int64_t, int64_t, int64_t, int,    \
                                          const FusedParams<T>&, BatchMask, cudaStream_t);    \
  template bool ct3_axis0_stiffness<T, 3>(int, cplx<T>*, int64_t, int64_t, int64_t, int,    \
                                          const FusedParams<T>&, BatchMask, cudaStream_t);    \
  template void ct3_set_smem_attrs_t<T>(size_t);

#define BRI17_CT_INSTANTIATE(T)                                                             \
  template bool ct_rows_r2c<T>(int, const typename IoOf<T>::type*, cplx<T>*, int64_t, int,  \
                               const cplx<T>*, BatchMask, cudaStream_t);                   \
  template bool ct_rows_c2r<T>(int, const cplx<T>*, typename IoOf<T>::type*, int64_t, int,  \
                               const cplx<T>*, BatchMask, cudaStream_t);                   \
  template bool ct_axis_c2c<T, false>(int, cplx<T>*, int64_t, int64_t, const cplx<T>*,      \
                                      BatchMask, cudaStream_t);                             \
  template bool ct_axis_c2c<T, true>(int, cplx<T>*, int64_t, int64_t, const cplx<T>*,       \
                                     BatchMask, cudaStream_t);                              \
  template bool ct_axis0_stiffness<T, 2>(int, cplx<T>*, int64_t, int64_t, int64_t, int,     \
                                         const FusedParams<T>&, BatchMask, cudaStream_t);   \
  template bool ct_axis0_stiffness<T, 3>(int, cplx<T>*, int64_t, int64_t, int64_t, int,     \
                                         const FusedParams<T>&, BatchMask, cudaStream_t);   \
  template bool ct_axis0_stiffness_staged<T, 2>(int, cplx<T>*, int64_t, int64_t, int64_t,   \
                                                int, const FusedParams<T>&, BatchMask,      \
                                                cudaStream_t);                              \
  template bool ct_axis0_stiffness_staged<T, 3>(int, cplx<T>*, int64_t, int64_t, int64_t,   \
                                                int, const FusedParams<T>&, BatchMask,      \
                                                cudaStream_t);                              \
  template void ct_set_smem_attrs_t<T>(size_t);

}  // namespace bri17gb
