// passes_p2.cuh -- the operator's FFT passes for power-of-two axis lengths,
// on the register-resident engine of fft8.cuh.  Same data layout, same
// results (to rounding) and same pass structure as passes.cuh, which keeps
// serving every other length.
#pragma once

#include <type_traits>

#include "df64.cuh"
#include "fft8.cuh"
#include "fft8_ct.cuh"
#include "passes.cuh"
#include "pdl.cuh"
#include "reduce.cuh"
#include "tma.cuh"

namespace bri17gb {

// Engine policies: the kernels below take either the runtime-plan engine
// (any power-of-two length) or a compile-time-length engine.
// load_tw fills the kernel's shared twiddle table from the natural global
// table (`count` entries read with stride `tws` by the transform); run then
// takes that shared table.  The runtime engine copies the natural table;
// the compile-time engine lays out per-stage tables (fftE_ct_twiddles), so
// consecutive butterflies read consecutive entries -- except in float pairs,
// whose transforms are bound by arithmetic, not by shared-memory banks, and
// keep the cheaper natural copy.  stage<S>() tells which table run reads.
struct RtEng {
  static constexpr int E = 8;
  static constexpr int kTT = 0;  // threads per line: known at run time only
  template <typename S>
  static constexpr bool stage() {
    return false;
  }
  Plan8 p;
  __device__ __forceinline__ int n() const { return p.n; }
  __device__ __forceinline__ int T() const { return p.T; }
  template <typename S>
  __device__ __forceinline__ void load_tw(cplx<S>* dst, const cplx<S>* __restrict__ src,
                                          int count, int tws) const {
    for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = src[i];
  }
  template <typename S, bool INV>
  __device__ __forceinline__ void run(cplx<S> (&v)[8], cplx<S>* buf, int t,
                                      const cplx<S>* __restrict__ tw, int tws) const {
    fft8_line<S, INV>(v, buf, t, p, tw, tws);
  }
};

template <int N, int EE = 8>
struct CtEng {
  static constexpr int E = EE;
  static constexpr int kTT = N / EE;
  template <typename S>
  static constexpr bool stage() {
    return !std::is_same<S, df64>::value;
  }
  __device__ __forceinline__ constexpr int n() const { return N; }
  __device__ __forceinline__ constexpr int T() const { return N / EE; }
  template <typename S>
  __device__ __forceinline__ void load_tw(cplx<S>* dst, const cplx<S>* __restrict__ src,
                                          int count, int tws) const {
    if constexpr (stage<S>())
      fftE_ct_twiddles<S, N, EE>(dst, src, tws, threadIdx.x, blockDim.x);
    else
      for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = src[i];
  }
  template <typename S, bool INV>
  __device__ __forceinline__ void run(cplx<S> (&v)[EE], cplx<S>* buf, int t,
                                      const cplx<S>* __restrict__ tw, int tws) const {
    if constexpr (stage<S>())
      fftE_ct<S, N, EE, INV>(v, buf, t, tw);
    else
      fftE_ct_nat<S, N, EE, INV>(v, buf, t, tw, tws);
  }
  // The same transform with the exchanges at every BS-th entry of `buf`
  // (the line's column of a tile laid out [element][BS lines]); natural
  // twiddle table only.  The first exchange writes `buf` without a barrier
  // before it: the caller makes sure every thread of the line has read what
  // it needs from there.
  template <typename S, bool INV, int BS>
  __device__ __forceinline__ void run_strided(cplx<S> (&v)[EE], cplx<S>* buf, int t,
                                              const cplx<S>* __restrict__ tw, int tws) const {
    static_assert(!stage<S>() && BS > 0, "strided exchanges read the natural table");
    fftE_ct_nat<S, N, EE, INV, BS>(v, buf, t, tw, tws);
  }
};

// Compile-time engine for lengths N = 3 * 2^k (fft8_ct.cuh PE3): twelve
// elements per thread, per-stage twiddle tables (FP32 and FP64 only; the
// float-pair passes are power-of-two only).
template <int N>
struct CtEng3 {
  using P = PE3<N>;
  static constexpr int E = P::kE;
  static constexpr int kTT = P::T;
  template <typename S>
  static constexpr bool stage() {
    return true;
  }
  __device__ __forceinline__ constexpr int n() const { return N; }
  __device__ __forceinline__ constexpr int T() const { return P::T; }
  template <typename S>
  __device__ __forceinline__ void load_tw(cplx<S>* dst, const cplx<S>* __restrict__ src,
                                          int count, int tws) const {
    fftP_twiddles<S, P>(dst, src, tws, threadIdx.x, blockDim.x);
  }
  template <typename S, bool INV>
  __device__ __forceinline__ void run(cplx<S> (&v)[E], cplx<S>* buf, int t,
                                      const cplx<S>* __restrict__ tw, int tws) const {
    fftP<S, P, INV>(v, buf, t, tw);
  }
};

constexpr int kP2Threads = 256;
constexpr int kP2FusedThreads = 128;

// Resident CTAs per SM that the forward row pass asks the register
// allocator for: FP32 fits 32 registers (eight 256-thread CTAs, the whole
// SM; 40 registers and six CTAs measured 79 -> 86 us at 256^3), float pairs
// 64 (four); FP64 is bound by the FP64 pipe and takes what the compiler
// picks.  With twelve elements per thread (lengths 3 * 2^k) 64 registers
// (FP32) and 128 (FP64).  The inverse row pass keeps the compiler's choice
// (FP32: 40 registers; capped at 32 it spills and measured 84 -> 89 us at
// 256^3).
template <typename T, int E = 8>
struct RowCtas {
  static constexpr bool kF32 = std::is_same<T, float>::value;
  static constexpr int value = E != 8 ? (kF32 ? 4 : 2)
                               : kF32 ? 8
                               : std::is_same<T, df64>::value ? 4
                                                              : 1;
};

// Warp shuffle of a complex value (float, double or float pair).
template <typename T>
__device__ __forceinline__ cplx<T> shfl_cplx(unsigned lanes, cplx<T> v, int src) {
  if constexpr (std::is_same<T, df64>::value) {
    cplx<T> r;
    r.x = df64(__shfl_sync(lanes, v.x.hi, src), __shfl_sync(lanes, v.x.lo, src));
    r.y = df64(__shfl_sync(lanes, v.y.hi, src), __shfl_sync(lanes, v.y.lo, src));
    return r;
  } else {
    return mk<T>(__shfl_sync(lanes, v.x, src), __shfl_sync(lanes, v.y, src));
  }
}

// The half-spectrum split of a row of m = TT E complex points held as
// v[q] = Z[t + TT q] (TT threads per row, a power of two <= 32, so a row
// lies in one warp) needs Z[(m - k) mod m] beside each Z[k]:
// for t > 0 that is element E-1-q of the row's thread TT - t, for t = 0 its
// own element (E - q) mod E.  mirror_lane gives the source lane of the
// shuffle and warp_lanes the lanes present in the calling thread's warp
// (the last warp of a small CTA may be partial; rows never straddle it).
template <int TT>
__device__ __forceinline__ int mirror_lane(int t) {
  const int lane = threadIdx.x & 31;
  return (lane & ~(TT - 1)) | ((TT - t) & (TT - 1));
}
__device__ __forceinline__ unsigned warp_lanes() {
  const int present = (int)blockDim.x - (int)(threadIdx.x & ~31u);
  return present >= 32 ? 0xffffffffu : ((1u << present) - 1u);
}

// Last axis, forward (n = 2m, m a power of two >= 8): rows of n reals ->
// n/2+1 complex.  T = m/8 threads per row, RB rows per CTA.
template <typename T, class Eng>
__global__ void __launch_bounds__(kP2Threads, RowCtas<T, Eng::E>::value)
    rows_r2c_p2(const typename IoOf<T>::type* __restrict__ x, cplx<T>* __restrict__ X,
                int64_t nrows, int H, Eng pm, const cplx<T>* __restrict__ tw_g, int RB,
                int pitch, BatchMask mask) {
  using Io = typename IoOf<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = pm.n(), n = 2 * m, TT = pm.T();
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* twh = tw + n;        // W_n^k / 2, k in [0, m]
  cplx<T>* bufs = twh + m + 1;
  const int64_t row0 = (int64_t)blockIdx.x * RB;
  const int t = threadIdx.x % TT, rb = threadIdx.x / TT;
  const int64_t row = row0 + rb;
  const bool valid = rb < RB && row < nrows;
  pdl_launch_dependents<T>();
  pm.template load_tw<T>(tw, tw_g, n, 2);
  for (int i = threadIdx.x; i <= m; i += blockDim.x) {
    const cplx<T> w = tw_g[i];
    twh[i] = mk<T>(T(0.5) * w.x, T(0.5) * w.y);
  }
  pdl_wait();
  if (mask.skip(row0)) return;
  cplx<T> v[Eng::E];
  const cplx<Io>* xc = reinterpret_cast<const cplx<Io>*>(x) + row * m;
#pragma unroll
  for (int q = 0; q < Eng::E; q++) {
    if (valid) {
      const cplx<Io> w = xc[t + TT * q];
      v[q] = mk<T>(from_io<T>(w.x), from_io<T>(w.y));
    } else {
      v[q] = mk<T>(T(0), T(0));
    }
  }
  __syncthreads();
  cplx<T>* buf = bufs + rb * pitch;
  pm.template run<T, false>(v, buf, t, tw, 2);
  // Z_{m-k}: from the row's mirror thread by warp shuffles when a row lies
  // in one warp (every lane stays to the end: shuffles name whole rows),
  // else through the exchange buffer.
  constexpr bool kShfl = Eng::kTT > 0 && Eng::kTT <= 32;
  unsigned lanes = 0;
  int src = 0;
  if constexpr (kShfl) {
    lanes = warp_lanes();
    src = mirror_lane<Eng::kTT>(t);
  } else {
#pragma unroll
    for (int q = 0; q < Eng::E; q++) buf[pad16(t + TT * q)] = v[q];
    __syncthreads();
    if (!valid) return;
  }
  cplx<T>* out = X + row * H;
  // X_k = (A + W D) / 2 with A = Z_k + conj(Z_{m-k}), D = -i (Z_k -
  // conj(Z_{m-k})), W = W_n^k; the 1/2 lives in the twh table and one fused
  // multiply-add per part.
  if constexpr (kShfl) {
    // A_{m-k} = conj(A_k), D_{m-k} = conj(D_k) and W^{m-k} = -conj(W^k), so
    // X_{m-k} = conj(A_k/2 - W D_k/2): each thread forms both outputs of
    // its pairs k < m/2 (for k = 0 the pair is X_0 and X_m), half the
    // arithmetic and half the shuffles of one output per element.
    constexpr int EH = Eng::E / 2;
#pragma unroll
    for (int q = 0; q < EH; q++) {
      const int k = t + TT * q;
      const cplx<T> o = shfl_cplx<T>(lanes, v[Eng::E - 1 - q], src);
      const cplx<T> zk = v[q];
      const cplx<T> zm = t == 0 ? v[(Eng::E - q) % Eng::E] : o;
      const cplx<T> A = mk<T>(zk.x + zm.x, zk.y - zm.y);
      const cplx<T> D = mk<T>(zk.y + zm.y, zm.x - zk.x);
      const cplx<T> WD = cmul<T>(twh[k], D);
      if (valid) {
        out[k] = mk<T>(fma(T(0.5), A.x, WD.x), fma(T(0.5), A.y, WD.y));
        out[m - k] = mk<T>(fma(T(0.5), A.x, -WD.x), -fma(T(0.5), A.y, -WD.y));
      }
    }
    if (valid && t == 0) {  // k = m/2, its own mirror
      const cplx<T> z = v[EH];
      const cplx<T> A = mk<T>(z.x + z.x, z.y - z.y);
      const cplx<T> D = mk<T>(z.y + z.y, z.x - z.x);
      const cplx<T> WD = cmul<T>(twh[m / 2], D);
      out[m / 2] = mk<T>(fma(T(0.5), A.x, WD.x), fma(T(0.5), A.y, WD.y));
    }
  } else {
#pragma unroll
    for (int q = 0; q < Eng::E; q++) {
      const int k = t + TT * q;
      const cplx<T> zk = v[q];
      const cplx<T> zm = buf[pad16((m - k) & (m - 1))];
      const cplx<T> A = mk<T>(zk.x + zm.x, zk.y - zm.y);
      const cplx<T> D = mk<T>(zk.y + zm.y, zm.x - zk.x);
      const cplx<T> WD = cmul<T>(twh[k], D);
      if (valid) out[k] = mk<T>(fma(T(0.5), A.x, WD.x), fma(T(0.5), A.y, WD.y));
    }
    if (valid && t == 0) out[m] = mk<T>(v[0].x - v[0].y, T(0));
  }
}

// Last axis, inverse: n/2+1 complex -> n reals (unnormalised).
template <typename T, class Eng>
__global__ void __launch_bounds__(kP2Threads)
    rows_c2r_p2(const cplx<T>* __restrict__ X, typename IoOf<T>::type* __restrict__ x,
                int64_t nrows, int H, Eng pm, const cplx<T>* __restrict__ tw_g, int RB,
                int pitch, BatchMask mask) {
  using Io = typename IoOf<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int m = pm.n(), n = 2 * m, TT = pm.T();
  // Natural table (the split step reads W^k) and, for the compile-time
  // engine, the transform's per-stage tables after it.
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* stw = tw + n;
  cplx<T>* bufs = stw + (Eng::template stage<T>() ? m : 0);
  const int64_t row0 = (int64_t)blockIdx.x * RB;
  const int t = threadIdx.x % TT, rb = threadIdx.x / TT;
  const int64_t row = row0 + rb;
  const bool valid = rb < RB && row < nrows;
  pdl_launch_dependents<T>();
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = tw_g[i];
  if constexpr (Eng::template stage<T>()) pm.template load_tw<T>(stw, tw_g, n, 2);
  __syncthreads();
  pdl_wait();
  if (mask.skip(row0)) return;
  cplx<T> v[Eng::E];
  const cplx<T>* in = X + row * H;
  constexpr bool kShfl = Eng::kTT > 0 && Eng::kTT <= 32;
  if constexpr (kShfl) {
    // Each thread loads its own X_k once; X_{m-k} comes from the row's
    // mirror thread by warp shuffles (X_m, which no thread holds, is loaded
    // by thread 0 of the row).
    const cplx<T> zero = mk<T>(T(0), T(0));
    cplx<T> w[Eng::E];
#pragma unroll
    for (int q = 0; q < Eng::E; q++) w[q] = valid ? in[t + TT * q] : zero;
    const cplx<T> wm = (valid && t == 0) ? in[m] : zero;
    const unsigned lanes = warp_lanes();
    const int src = mirror_lane<Eng::kTT>(t);
    // Z_k = A + i conj(W^k) D with A = X_k + conj(X_{m-k}), D = X_k -
    // conj(X_{m-k}); as in the forward pass Z_{m-k} = conj(A - i conj(W^k)
    // D), so each thread forms the pair of its k < m/2 and hands Z_{m-k} to
    // the mirror thread, which holds it as element E-1-q (thread 0 holds its
    // own mirrors, Z_{m-k} as element E-q, and Z_{m/2}).
    constexpr int EH = Eng::E / 2;
    cplx<T> zmir[EH];
#pragma unroll
    for (int q = 0; q < EH; q++) {
      const int k = t + TT * q;
      const cplx<T> o = shfl_cplx<T>(lanes, w[Eng::E - 1 - q], src);
      const cplx<T> xk = w[q];
      const cplx<T> xm = t != 0 ? o : (q == 0 ? wm : w[(Eng::E - q) % Eng::E]);
      const cplx<T> A = mk<T>(xk.x + xm.x, xk.y - xm.y);
      const cplx<T> D = mk<T>(xk.x - xm.x, xk.y + xm.y);
      const cplx<T> Bv = cmulc<T>(D, tw[k]);
      v[q] = mk<T>(A.x - Bv.y, A.y + Bv.x);
      zmir[q] = mk<T>(A.x + Bv.y, Bv.x - A.y);
    }
    cplx<T> zhalf = zero;
    if (t == 0) {  // k = m/2, its own mirror
      const cplx<T> x = w[EH];
      const cplx<T> A = mk<T>(x.x + x.x, x.y - x.y);
      const cplx<T> D = mk<T>(x.x - x.x, x.y + x.y);
      const cplx<T> Bv = cmulc<T>(D, tw[m / 2]);
      zhalf = mk<T>(A.x - Bv.y, A.y + Bv.x);
    }
#pragma unroll
    for (int q = 0; q < EH; q++) {
      const cplx<T> r = shfl_cplx<T>(lanes, zmir[q], src);
      // Element E-1-q: the mirror's Z_{m-k}; for thread 0 its own Z_{m/2}
      // (q = EH-1) or the mirror of its element E-1-q.
      const int j = Eng::E - 1 - q;
      v[j] = t != 0 ? r : (j == EH ? zhalf : zmir[(Eng::E - j) % EH]);
    }
  } else {
#pragma unroll
    for (int q = 0; q < Eng::E; q++) {
      const int k = t + TT * q;
      if (valid) {
        const cplx<T> xk = in[k];
        const cplx<T> xm = in[m - k];
        const cplx<T> A = mk<T>(xk.x + xm.x, xk.y - xm.y);
        const cplx<T> D = mk<T>(xk.x - xm.x, xk.y + xm.y);
        const cplx<T> Bv = cmulc<T>(D, tw[k]);
        v[q] = mk<T>(A.x - Bv.y, A.y + Bv.x);
      } else {
        v[q] = mk<T>(T(0), T(0));
      }
    }
  }
  pm.template run<T, true>(v, bufs + rb * pitch, t, Eng::template stage<T>() ? stw : tw, 2);
  if (!valid) return;
  cplx<Io>* xc = reinterpret_cast<cplx<Io>*>(x) + row * m;
#pragma unroll
  for (int q = 0; q < Eng::E; q++) xc[t + TT * q] = mk<Io>(to_io<T>(v[q].x), to_io<T>(v[q].y));
}

// Middle axis: complex [A][n][B], lines along n.  The A * B lines are
// numbered plane-major (line = a B + b) and dealt out TB consecutive lines
// per CTA, consecutive threads on consecutive lines (coalesced; a CTA may
// straddle two planes).  With B = n_last/2 + 1 odd, a grid over b alone
// would leave one CTA per plane holding a single line (a fifth of the
// CTAs at 128^3, a ninth at 256^3) running full transforms on zeros.
template <typename T, bool INV, class Eng>
__global__ void __launch_bounds__(kP2Threads)
    axis_c2c_p2(cplx<T>* __restrict__ X, int64_t B, int64_t nlines, int TB, Eng p,
                const cplx<T>* __restrict__ tw_g, int pitch, BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = p.n();
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bufs = tw + n;
  const int tb = threadIdx.x % TB, t = threadIdx.x / TB;
  const int64_t line = (int64_t)blockIdx.x * TB + tb;
  const int64_t a = line / B;
  bool valid = line < nlines;
  cplx<T>* base = X + a * n * B + (line - a * B);
  pdl_launch_dependents<T>();
  p.template load_tw<T>(tw, tw_g, n, 1);
  pdl_wait();
  if (mask.flags) {
    valid = valid && !mask.skip(a);
    if (!__syncthreads_or(valid)) return;
  }
  cplx<T> v[Eng::E];
#pragma unroll
  for (int q = 0; q < Eng::E; q++)
    v[q] = valid ? base[(int64_t)(t + p.T() * q) * B] : mk<T>(T(0), T(0));
  __syncthreads();
  p.template run<T, INV>(v, bufs + tb * pitch, t, tw, 1);
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < Eng::E; q++) base[(int64_t)(t + p.T() * q) * B] = v[q];
}

// Per-line coefficients of K(k) for the modes of one spectrum line (fixed
// axis-1/axis-2 wavenumbers), from Hooke::modal_stiffness
// (include/bri17/bri17.hpp:258-288): with H00 = phi0 chi1 chi2, H11 =
// chi0 phi1 chi2, H22 = chi0 chi1 phi2, K_ii = s H_ii + mu (H00 + H11 + H22)
// and K_ij = s psi_i psi_j chi_l, every entry is linear in the mode's
// axis-0 factors phi0, chi0, psi0 with per-line coefficients (material
// included), so a mode's K(k) costs 8 products and sums (3D) instead of 14.
// The fused operator holds the oracle's 1e-12 bound either way; the per-mode
// entry points (modal_stiffness_kernel) keep the reference's operation
// order.
template <typename T>
struct LineFactors {
  T g00, h00;  // K00 = phi0 g00 + chi0 h00
  T g11;       // mu H00 / phi0, shared by K11 and K22
  T h11, h22;  // K11 = chi0 h11 + phi0 g11, K22 = chi0 h22 + phi0 g11
  T spc, scp;  // K01 = psi0 spc, K02 = psi0 scp
  T spp;       // K12 = chi0 spp
};

template <typename T, int DIM>
__device__ __forceinline__ LineFactors<T> line_factors(T phi1, T chi1, T psi1, T phi2, T chi2,
                                                      T psi2, T s, T mu) {
  LineFactors<T> f;
  const T smu = s + mu;
  if constexpr (DIM == 3) {
    const T c12 = chi1 * chi2, a1 = phi1 * chi2, a2 = chi1 * phi2;
    f.g00 = smu * c12;
    f.h00 = mu * (a1 + a2);
    f.g11 = mu * c12;
    f.h11 = fma(s, a1, f.h00);
    f.h22 = fma(s, a2, f.h00);
    f.spc = s * (psi1 * chi2);
    f.scp = s * (chi1 * psi2);
    f.spp = s * (psi1 * psi2);
  } else {
    // H00 = phi0 chi1, H11 = chi0 phi1.
    f.g00 = smu * chi1;
    f.h00 = mu * phi1;
    f.g11 = mu * chi1;
    f.h11 = smu * phi1;
    f.h22 = T(0);
    f.spc = s * psi1;
    f.scp = T(0);
    f.spp = T(0);
  }
  return f;
}

template <typename T, int DIM>
__device__ __forceinline__ void stiffness_lf(T phi0, T chi0, T psi0, const LineFactors<T>& f,
                                             cplx<T>* u) {
  const T K00 = fma(chi0, f.h00, phi0 * f.g00);
  const T mg = phi0 * f.g11;
  const T K11 = fma(chi0, f.h11, mg);
  const T K01 = psi0 * f.spc;
  if constexpr (DIM == 3) {
    const T K22 = fma(chi0, f.h22, mg);
    const T K02 = psi0 * f.scp;
    const T K12 = chi0 * f.spp;
    const cplx<T> u0 = u[0], u1 = u[1], u2 = u[2];
    if constexpr (std::is_same<T, df64>::value) {
      // Float pairs: each entry one fused three-term sum (df_dot3).
      u[0] = mk<T>(df_dot3(K00, u0.x, K01, u1.x, K02, u2.x),
                   df_dot3(K00, u0.y, K01, u1.y, K02, u2.y));
      u[1] = mk<T>(df_dot3(K01, u0.x, K11, u1.x, K12, u2.x),
                   df_dot3(K01, u0.y, K11, u1.y, K12, u2.y));
      u[2] = mk<T>(df_dot3(K02, u0.x, K12, u1.x, K22, u2.x),
                   df_dot3(K02, u0.y, K12, u1.y, K22, u2.y));
    } else {
      u[0] = mk<T>(K00 * u0.x + K01 * u1.x + K02 * u2.x, K00 * u0.y + K01 * u1.y + K02 * u2.y);
      u[1] = mk<T>(K01 * u0.x + K11 * u1.x + K12 * u2.x, K01 * u0.y + K11 * u1.y + K12 * u2.y);
      u[2] = mk<T>(K02 * u0.x + K12 * u1.x + K22 * u2.x, K02 * u0.y + K12 * u1.y + K22 * u2.y);
    }
  } else {
    const cplx<T> u0 = u[0], u1 = u[1];
    if constexpr (std::is_same<T, df64>::value) {
      u[0] = mk<T>(df_dot2(K00, u0.x, K01, u1.x), df_dot2(K00, u0.y, K01, u1.y));
      u[1] = mk<T>(df_dot2(K01, u0.x, K11, u1.x), df_dot2(K01, u0.y, K11, u1.y));
    } else {
      u[0] = mk<T>(K00 * u0.x + K01 * u1.x, K00 * u0.y + K01 * u1.y);
      u[1] = mk<T>(K01 * u0.x + K11 * u1.x, K01 * u0.y + K11 * u1.y);
    }
  }
}

// Axis 0, fused stiffness: forward DFT of the DIM components along axis 0,
// K(k) u(k) in registers, inverse DFT, in place (as axis0_fused with
// kModeStiffness).
template <typename T, int DIM, class Eng>
__global__ void __launch_bounds__(kP2FusedThreads)
    axis0_stiffness_p2(cplx<T>* __restrict__ X, int64_t P, int64_t cstride,
                       int64_t bstride, int TB, int pitch, Eng p0, FusedParams<T> fp,
                       BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n0 = p0.n();
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bufs = tw + n0;
  const int tb = threadIdx.x % TB, t = threadIdx.x / TB;
  const int64_t b = (int64_t)blockIdx.x * TB + tb;
  const bool valid = b < P;
  cplx<T>* base = X + (int64_t)blockIdx.y * bstride + b;
  pdl_launch_dependents<T>();
  p0.template load_tw<T>(tw, fp.tab.tw[0], n0, 1);
  pdl_wait();
  if (mask.skip(blockIdx.y)) return;
  T s = fp.s, mu = fp.mu;
  if (fp.mat) {
    s = fp.mat[2 * blockIdx.y];
    mu = fp.mat[2 * blockIdx.y + 1];
  }
  cplx<T> v[DIM][Eng::E];
  cplx<T>* buf = bufs + tb * pitch;
#pragma unroll
  for (int c = 0; c < DIM; c++)
#pragma unroll
    for (int q = 0; q < Eng::E; q++)
      v[c][q] = valid ? base[c * cstride + (int64_t)(t + p0.T() * q) * P]
                      : mk<T>(T(0), T(0));
  __syncthreads();
#pragma unroll
  for (int c = 0; c < DIM; c++) p0.template run<T, false>(v[c], buf, t, tw, 1);
  int k1 = 0, k2 = 0;
  if (valid) {
    if constexpr (DIM == 3) {
      k1 = (int)(b / fp.H);
      k2 = (int)(b - (int64_t)k1 * fp.H);
    } else {
      k1 = (int)b;
    }
  }
  const T phi1 = ldg_val(fp.tab.kphi[1] + k1), chi1 = ldg_val(fp.tab.kchi[1] + k1),
          psi1 = ldg_val(fp.tab.kpsi[1] + k1);
  T phi2 = T(1), chi2 = T(1), psi2 = T(1);
  if constexpr (DIM == 3) {
    phi2 = ldg_val(fp.tab.kphi[2] + k2);
    chi2 = ldg_val(fp.tab.kchi[2] + k2);
    psi2 = ldg_val(fp.tab.kpsi[2] + k2);
  }
  // Per-line products of the axis-1/axis-2 factors (2D: axis 1 only).
  LineFactors<T> lf = line_factors<T, DIM>(phi1, chi1, psi1, phi2, chi2, psi2, s, mu);
#pragma unroll
  for (int q = 0; q < Eng::E; q++) {
    const int k0 = t + p0.T() * q;
    const T phi0 = ldg_val(fp.tab.kphi[0] + k0), chi0 = ldg_val(fp.tab.kchi[0] + k0),
            psi0 = ldg_val(fp.tab.kpsi[0] + k0);
    cplx<T> u[DIM];
#pragma unroll
    for (int c = 0; c < DIM; c++) u[c] = v[c][q];
    stiffness_lf<T, DIM>(phi0, chi0, psi0, lf, u);
#pragma unroll
    for (int c = 0; c < DIM; c++) v[c][q] = u[c];
  }
#pragma unroll
  for (int c = 0; c < DIM; c++) p0.template run<T, true>(v[c], buf, t, tw, 1);
  if (!valid) return;
#pragma unroll
  for (int c = 0; c < DIM; c++)
#pragma unroll
    for (int q = 0; q < Eng::E; q++) base[c * cstride + (int64_t)(t + p0.T() * q) * P] = v[c][q];
}

}  // namespace bri17gb

namespace bri17gb {

// Axis 0, fused stiffness, shared-memory staged: the same computation as
// axis0_stiffness_p2 with one component in registers at a time.  Each
// component's forward transform is parked in shared memory at the thread's
// own positions (no barrier needed: a thread reads back only what it wrote),
// K(k) u(k) runs from there, and the inverse transforms read it back.  Half
// the registers of the register-resident form, so twice the warps per SM.
template <typename T, int DIM, class Eng>
__global__ void __launch_bounds__(kP2Threads)
    axis0_stiffness_staged(cplx<T>* __restrict__ X, int64_t P, int64_t cstride,
                           int64_t bstride, int TB, int pitch, Eng p0, FusedParams<T> fp,
                           BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n0 = p0.n();
  // Staged lines are only read and written at a thread's own positions,
  // lanes stepping across the TB lines first: their pitch staggers lines by
  // 32 / TB elements modulo one 128-byte bank row.
  const int spitch = stash_pitch(n0, TB, (int)sizeof(cplx<T>));
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* exch = tw + n0;                      // TB exchange lines
  cplx<T>* stash = exch + (size_t)TB * pitch;   // DIM x TB staged lines
  const int tb = threadIdx.x % TB, t = threadIdx.x / TB;
  const int64_t b = (int64_t)blockIdx.x * TB + tb;
  const bool valid = b < P;
  cplx<T>* base = X + (int64_t)blockIdx.y * bstride + b;
  pdl_launch_dependents<T>();
  p0.template load_tw<T>(tw, fp.tab.tw[0], n0, 1);
  pdl_wait();
  if (mask.skip(blockIdx.y)) return;
  T s = fp.s, mu = fp.mu;
  if (fp.mat) {
    s = fp.mat[2 * blockIdx.y];
    mu = fp.mat[2 * blockIdx.y + 1];
  }
  __syncthreads();
  cplx<T>* buf = exch + tb * pitch;
  cplx<T> v[Eng::E];
#pragma unroll 1
  for (int c = 0; c < DIM; c++) {
#pragma unroll
    for (int q = 0; q < Eng::E; q++)
      v[q] = valid ? base[c * cstride + (int64_t)(t + p0.T() * q) * P] : mk<T>(T(0), T(0));
    p0.template run<T, false>(v, buf, t, tw, 1);
    cplx<T>* st = stash + ((size_t)c * TB + tb) * spitch;
#pragma unroll
    for (int q = 0; q < Eng::E; q++) st[t + p0.T() * q] = v[q];
  }
  int k1 = 0, k2 = 0;
  if (valid) {
    if constexpr (DIM == 3) {
      k1 = (int)(b / fp.H);
      k2 = (int)(b - (int64_t)k1 * fp.H);
    } else {
      k1 = (int)b;
    }
  }
  const T phi1 = ldg_val(fp.tab.kphi[1] + k1), chi1 = ldg_val(fp.tab.kchi[1] + k1),
          psi1 = ldg_val(fp.tab.kpsi[1] + k1);
  T phi2 = T(1), chi2 = T(1), psi2 = T(1);
  if constexpr (DIM == 3) {
    phi2 = ldg_val(fp.tab.kphi[2] + k2);
    chi2 = ldg_val(fp.tab.kchi[2] + k2);
    psi2 = ldg_val(fp.tab.kpsi[2] + k2);
  }
  const LineFactors<T> lf = line_factors<T, DIM>(phi1, chi1, psi1, phi2, chi2, psi2, s, mu);
#pragma unroll 2
  for (int q = 0; q < Eng::E; q++) {
    const int k0 = t + p0.T() * q;
    const T phi0 = ldg_val(fp.tab.kphi[0] + k0), chi0 = ldg_val(fp.tab.kchi[0] + k0),
            psi0 = ldg_val(fp.tab.kpsi[0] + k0);
    cplx<T> u[DIM];
#pragma unroll
    for (int c = 0; c < DIM; c++) u[c] = stash[((size_t)c * TB + tb) * spitch + k0];
    stiffness_lf<T, DIM>(phi0, chi0, psi0, lf, u);
#pragma unroll
    for (int c = 0; c < DIM; c++) stash[((size_t)c * TB + tb) * spitch + k0] = u[c];
  }
#pragma unroll 1
  for (int c = 0; c < DIM; c++) {
    const cplx<T>* st = stash + ((size_t)c * TB + tb) * spitch;
#pragma unroll
    for (int q = 0; q < Eng::E; q++) v[q] = st[t + p0.T() * q];
    p0.template run<T, true>(v, buf, t, tw, 1);
    if (valid) {
#pragma unroll
      for (int q = 0; q < Eng::E; q++) base[c * cstride + (int64_t)(t + p0.T() * q) * P] = v[q];
    }
  }
}

// p.Kp of a CG iteration from the stiffness pass, by Parseval: with the
// unnormalised forward transform and K(k) carrying the inverse's 1/|N|,
// sum_x p(x) (K p)(x) = sum over the half spectrum of w Re(conj(p^) (K p)^),
// w = 1 on the k_last = 0 and Nyquist lines (even last axis) and 2 elsewhere.
// Each CTA reduces its threads' sums (`part`, already without w; `w` the
// line's weight) through `red` (9 doubles of shared memory) into one partial
// per CTA; the last CTA to finish adds the partials in index order (the
// result does not depend on the order the CTAs ran in), sets pq and
// alpha = rr / pq, or flags a breakdown when pq is not positive and finite,
// while the CG is active.  Every thread of the CTA calls it.
template <typename T>
__device__ __forceinline__ void cg_pq_reduce(float part, double w, const FusedParams<T>& fp,
                                             double* red) {
  const int nwarps = (int)(blockDim.x >> 5), lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double v = w * (double)part;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int* last = reinterpret_cast<int*>(red + 8);
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int i = 0; i < nwarps; i++) b += red[i];
    fp.cg_part[blockIdx.x] = b;
    __threadfence();
    const unsigned t = atomicAdd(&fp.cg->counter, 1u);
    *last = t == gridDim.x - 1;
  }
  __syncthreads();
  if (*last) {
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += __ldcg(fp.cg_part + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncthreads();
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int i = 0; i < nwarps; i++) tot += red[i];
      CgState* st = fp.cg;
      if (st->active) {
        st->pq = tot;
        if (!(tot > 0.0) || !isfinite(tot)) {
          st->flag = BRI17_ERR_BREAKDOWN;
          st->active = 0;
        } else {
          st->alpha = st->rr / tot;
        }
      }
      st->counter = 0u;
    }
  }
}

// Bounded mbarrier waits that ran out in this translation unit's TMA kernels.
static __device__ int g_tma_timeouts;
// Limit of the first wait on a tile's copies (ns of global time).
static __device__ unsigned long long g_tma_wait_limit_ns = kWaitLimitNs;

// Axis 0, fused stiffness, TMA-staged (3D): the CTA's tile -- TB consecutive
// lines of all DIM components, n0 rows each, laid out [c][k0][line] in shared
// memory -- arrives by tensor copies that one thread issues all at once (one
// per component and 256 rows), so the whole tile's HBM traffic is in flight
// together and no registers wait on it.  The transforms and K(k) u(k) run
// between the tile and registers at each thread's own positions (as in the
// staged form) and tensor copies write the tile back.  Lines past P read as
// zeros and their stores are clipped by the copy engine.  The map views the
// spectrum as [plane = batch entry * DIM + component][k0][2 P reals].
//
// KEEP selects where the spectra wait between the transforms: false parks
// each component's forward transform in the tile (one component in
// registers at a time); true keeps all DIM components in registers from the
// forward transforms through K(k) u(k) to the inverse ones (fewer
// shared-memory round trips, more registers).
//
// XS > 0 (float pairs, TB = XS lines of 128 bytes per tile row): a
// component's transforms exchange through the component's own slot of the
// tile -- element p of line tb at row p, column tb -- instead of a separate
// exchange buffer.  The slot's values are in registers while it is
// transformed, so it is free; one barrier after the loads keeps the first
// exchange from overwriting values other threads of the line have not
// loaded yet.  A warp's lanes cover the TB lines of four rows, so each
// access takes the four wavefronts its 512 bytes need, and the CTA's shared
// memory shrinks by the exchange buffer (128^3: 69 -> 52 KB, four resident
// CTAs per SM instead of three).
template <typename T, int DIM, class Eng, bool KEEP, bool PQ = false, int XS = 0>
__global__ void __launch_bounds__(256)
    axis0_stiffness_tma(const __grid_constant__ CUtensorMap map, int64_t P, int TB, int pitch,
                        Eng p0, FusedParams<T> fp, BatchMask mask) {
  static_assert(DIM == 3, "three-dimensional grids only");
  static_assert(XS == 0 || (!KEEP && !PQ), "in-tile exchanges: staged compute only");
  extern __shared__ __align__(128) unsigned char smem_tma[];
  constexpr int kPer = (int)(sizeof(cplx<T>) / sizeof(T));  // map elements per complex
  const int n0 = p0.n();
  const int rows = n0 < 256 ? n0 : 256;  // box height (at most 256)
  cplx<T>* tile = reinterpret_cast<cplx<T>*>(smem_tma);
  cplx<T>* exch = tile + (size_t)DIM * n0 * TB;
  cplx<T>* tw = exch + (XS > 0 ? (size_t)0 : (size_t)TB * pitch);
  uint64_t* bar = reinterpret_cast<uint64_t*>(tw + n0);
  const int tb = threadIdx.x % TB, t = threadIdx.x / TB;
  const int64_t b = (int64_t)blockIdx.x * TB + tb;
  const int x0 = (int)((int64_t)blockIdx.x * TB * kPer);
  const int z = blockIdx.y;
  pdl_launch_dependents<T>();
  if (threadIdx.x == 0) mbar_init(bar, 1);
  p0.template load_tw<T>(tw, fp.tab.tw[0], n0, 1);
  pdl_wait();
  // A CTA that leaves early still takes its part in the p.Kp reduction (a
  // zero), so that the last CTA is found and the ticket counter returns to 0.
  double* red = reinterpret_cast<double*>(bar + 1);
  if (mask.skip(blockIdx.y)) {
    if constexpr (PQ) cg_pq_reduce<T>(0.f, 0.0, fp, red);
    return;
  }
  // The copy destinations must be 128-byte aligned, and in-tile exchanges
  // need TB = XS; the launch guarantees both, and a misplaced window skips
  // the CTA with an error count.
  if ((smem_addr(tile) & 127u) || (XS > 0 && TB != XS)) {
    if (threadIdx.x == 0) {
      atomicAdd(&g_tma_timeouts, 1);
      report_status(fp.status, 1);
    }
    if constexpr (PQ) cg_pq_reduce<T>(0.f, 0.0, fp, red);
    return;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(bar, (uint32_t)((size_t)DIM * n0 * TB * sizeof(cplx<T>)));
    for (int c = 0; c < DIM; c++)
      for (int r0 = 0; r0 < n0; r0 += rows)
        tma_load_3d(tile + ((size_t)c * n0 + r0) * TB, &map, x0, r0, z * DIM + c, bar);
  }
  T s = fp.s, mu = fp.mu;
  if (fp.mat) {
    s = fp.mat[2 * blockIdx.y];
    mu = fp.mat[2 * blockIdx.y + 1];
  }
  const bool valid = b < P;
  int k1 = 0, k2 = 0;
  if (valid) {
    k1 = (int)(b / fp.H);
    k2 = (int)(b - (int64_t)k1 * fp.H);
  }
  const T phi1 = ldg_val(fp.tab.kphi[1] + k1), chi1 = ldg_val(fp.tab.kchi[1] + k1),
          psi1 = ldg_val(fp.tab.kpsi[1] + k1);
  const T phi2 = ldg_val(fp.tab.kphi[2] + k2), chi2 = ldg_val(fp.tab.kchi[2] + k2),
          psi2 = ldg_val(fp.tab.kpsi[2] + k2);
  const LineFactors<T> lf = line_factors<T, DIM>(phi1, chi1, psi1, phi2, chi2, psi2, s, mu);
  // One second of global time per wait (g_tma_wait_limit_ns); a wait that
  // runs out is counted and reported to the handle, the tile is neither
  // transformed nor stored, and the CTA waits (bounded again, by
  // kWaitLimitNs) for its copies to land before leaving, so that no copy
  // writes shared memory after the CTA has left.
  const bool arrived = mbar_wait(bar, 0, g_tma_wait_limit_ns);
  if (__syncthreads_or(!arrived)) {
    if (threadIdx.x == 0) {
      atomicAdd(&g_tma_timeouts, 1);
      report_status(fp.status, 0);
      mbar_wait(bar, 0, kWaitLimitNs);
    }
    if constexpr (PQ) cg_pq_reduce<T>(0.f, 0.0, fp, red);
    return;
  }
  cplx<T>* buf = exch + tb * pitch;
  if constexpr (KEEP) {
    cplx<T> v[DIM][Eng::E];
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      const cplx<T>* tc = tile + (size_t)c * n0 * TB + tb;
#pragma unroll
      for (int q = 0; q < Eng::E; q++) v[c][q] = tc[(t + p0.T() * q) * TB];
      p0.template run<T, false>(v[c], buf, t, tw, 1);
    }
#pragma unroll
    for (int q = 0; q < Eng::E; q++) {
      const int k0 = t + p0.T() * q;
      const T phi0 = ldg_val(fp.tab.kphi[0] + k0), chi0 = ldg_val(fp.tab.kchi[0] + k0),
              psi0 = ldg_val(fp.tab.kpsi[0] + k0);
      cplx<T> u[DIM];
#pragma unroll
      for (int c = 0; c < DIM; c++) u[c] = v[c][q];
      stiffness_lf<T, DIM>(phi0, chi0, psi0, lf, u);
#pragma unroll
      for (int c = 0; c < DIM; c++) v[c][q] = u[c];
    }
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      p0.template run<T, true>(v[c], buf, t, tw, 1);
      cplx<T>* tc = tile + (size_t)c * n0 * TB + tb;
#pragma unroll
      for (int q = 0; q < Eng::E; q++) tc[(t + p0.T() * q) * TB] = v[c][q];
    }
  } else {
    // One component in registers at a time, the others parked in the tile.
    // FP32 (KL): the last component's forward transform stays in registers
    // through K(k) u(k) and is the first to be transformed back, which
    // spares it four shared-memory passes (park, K read, K write, reload):
    // 80 registers instead of 64, pass time 131 -> 129 us at 256^3 and
    // 268 -> 260 us at 512x512x128.  Float pairs keep every component in
    // the tile (their registers are the constraint: the same change made
    // that pass slower, 80 -> 92 us at 128^3).
    constexpr bool KL = std::is_same<T, float>::value;
    static_assert(!PQ || KL, "p.Kp by Parseval: FP32 only");
    static_assert(XS == 0 || !KL, "in-tile exchanges: float pairs only");
    float pq = 0.f;  // this thread's modes' Re(conj(p) . K p), PQ only
    cplx<T> v[Eng::E];
#pragma unroll 1
    for (int c = 0; c < DIM; c++) {
      cplx<T>* tc = tile + (size_t)c * n0 * TB + tb;
#pragma unroll
      for (int q = 0; q < Eng::E; q++) v[q] = tc[(t + p0.T() * q) * TB];
      if constexpr (XS > 0) {
        __syncthreads();
        p0.template run_strided<T, false, XS>(v, tc, t, tw, 1);
      } else {
        p0.template run<T, false>(v, buf, t, tw, 1);
      }
      if (!KL || c < DIM - 1) {
#pragma unroll
        for (int q = 0; q < Eng::E; q++) tc[(t + p0.T() * q) * TB] = v[q];
      }
    }
    if constexpr (KL) {
#pragma unroll
      for (int q = 0; q < Eng::E; q++) {
        const int k0 = t + p0.T() * q;
        const T phi0 = ldg_val(fp.tab.kphi[0] + k0), chi0 = ldg_val(fp.tab.kchi[0] + k0),
                psi0 = ldg_val(fp.tab.kpsi[0] + k0);
        cplx<T> u[DIM];
#pragma unroll
        for (int c = 0; c < DIM - 1; c++) u[c] = tile[((size_t)c * n0 + k0) * TB + tb];
        u[DIM - 1] = v[q];
        cplx<T> u0[DIM];
        if constexpr (PQ) {
#pragma unroll
          for (int c = 0; c < DIM; c++) u0[c] = u[c];
        }
        stiffness_lf<T, DIM>(phi0, chi0, psi0, lf, u);
        if constexpr (PQ) {
#pragma unroll
          for (int c = 0; c < DIM; c++) pq = fmaf(u0[c].x, u[c].x, fmaf(u0[c].y, u[c].y, pq));
        }
#pragma unroll
        for (int c = 0; c < DIM - 1; c++) tile[((size_t)c * n0 + k0) * TB + tb] = u[c];
        v[q] = u[DIM - 1];
      }
      if constexpr (PQ)
        cg_pq_reduce<T>(pq, valid ? (k2 == 0 || k2 == fp.H - 1 ? 1.0 : 2.0) : 0.0, fp, red);
    } else {
#pragma unroll 2
      for (int q = 0; q < Eng::E; q++) {
        const int k0 = t + p0.T() * q;
        const T phi0 = ldg_val(fp.tab.kphi[0] + k0), chi0 = ldg_val(fp.tab.kchi[0] + k0),
                psi0 = ldg_val(fp.tab.kpsi[0] + k0);
        cplx<T> u[DIM];
#pragma unroll
        for (int c = 0; c < DIM; c++) u[c] = tile[((size_t)c * n0 + k0) * TB + tb];
        stiffness_lf<T, DIM>(phi0, chi0, psi0, lf, u);
#pragma unroll
        for (int c = 0; c < DIM; c++) tile[((size_t)c * n0 + k0) * TB + tb] = u[c];
      }
    }
#pragma unroll 1
    for (int i = 0; i < DIM; i++) {
      const int c = KL ? (i == 0 ? DIM - 1 : i - 1) : i;
      cplx<T>* tc = tile + (size_t)c * n0 * TB + tb;
      if (!KL || i > 0) {
#pragma unroll
        for (int q = 0; q < Eng::E; q++) v[q] = tc[(t + p0.T() * q) * TB];
      }
      if constexpr (XS > 0) {
        // Also orders every thread's K(k) u(k) writes to this slot before
        // the first exchange.
        __syncthreads();
        p0.template run_strided<T, true, XS>(v, tc, t, tw, 1);
      } else {
        p0.template run<T, true>(v, buf, t, tw, 1);
      }
#pragma unroll
      for (int q = 0; q < Eng::E; q++) tc[(t + p0.T() * q) * TB] = v[q];
    }
  }
  fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int c = 0; c < DIM; c++)
      for (int r0 = 0; r0 < n0; r0 += rows)
        tma_store_3d(&map, x0, r0, z * DIM + c, tile + ((size_t)c * n0 + r0) * TB);
    tma_store_commit_and_wait();
  }
}

// The tensor-copy layout the TMA-staged axis-0 launcher needs (false: it
// declines, launching nothing).
template <typename T>
inline bool tma_layout_ok(const void* X, int64_t P, int64_t cstride, int64_t bstride, int n0) {
  constexpr int kPer = (int)(sizeof(cplx<T>) / sizeof(T));
  return (P * (int64_t)sizeof(cplx<T>)) % 16 == 0 && cstride == (int64_t)n0 * P &&
         bstride == 3 * cstride && reinterpret_cast<uintptr_t>(X) % 16 == 0 &&
         (int64_t)P * kPer < ((int64_t)1 << 31);
}

// Launchers of the compile-time-length kernels (passes_ct.cuh, instantiated
// in passes_ct_f32.cu / passes_ct_f64.cu).  Each picks its own block
// geometry and returns false, launching nothing, when the length has no
// compile-time instance.
template <typename T>
bool ct_rows_r2c(int m, const typename IoOf<T>::type* x, cplx<T>* X, int64_t nrows, int H,
                 const cplx<T>* tw, BatchMask mask, cudaStream_t st);
template <typename T>
bool ct_rows_c2r(int m, const cplx<T>* X, typename IoOf<T>::type* x, int64_t nrows, int H,
                 const cplx<T>* tw, BatchMask mask, cudaStream_t st);
template <typename T, bool INV>
bool ct_axis_c2c(int n, cplx<T>* X, int64_t B, int64_t nouter, const cplx<T>* tw,
                 BatchMask mask, cudaStream_t st);
template <typename T, int DIM>
bool ct_axis0_stiffness(int n0, cplx<T>* X, int64_t P, int64_t cstride, int64_t bstride,
                        int batch, const FusedParams<T>& fp, BatchMask mask,
                        cudaStream_t st);
template <typename T, int DIM>
bool ct_axis0_stiffness_staged(int n0, cplx<T>* X, int64_t P, int64_t cstride,
                               int64_t bstride, int batch, const FusedParams<T>& fp,
                               BatchMask mask, cudaStream_t st);
// Lengths 3 * 2^k (passes_ct3_f32.cu / passes_ct3_f64.cu, FP32 and FP64
// only): false, launching nothing, for lengths without an instance.
template <typename T>
bool ct3_rows_r2c(int m, const typename IoOf<T>::type* x, cplx<T>* X, int64_t nrows, int H,
                  const cplx<T>* tw, BatchMask mask, cudaStream_t st);
template <typename T>
bool ct3_rows_c2r(int m, const cplx<T>* X, typename IoOf<T>::type* x, int64_t nrows, int H,
                  const cplx<T>* tw, BatchMask mask, cudaStream_t st);
template <typename T, bool INV>
bool ct3_axis_c2c(int n, cplx<T>* X, int64_t B, int64_t nouter, const cplx<T>* tw,
                  BatchMask mask, cudaStream_t st);
template <typename T, int DIM>
bool ct3_axis0_stiffness(int n0, cplx<T>* X, int64_t P, int64_t cstride, int64_t bstride,
                         int batch, const FusedParams<T>& fp, BatchMask mask, cudaStream_t st);
template <typename T>
void ct3_set_smem_attrs_t(size_t max_smem);
// TMA-staged forms (FP32, 3D; `keep` as KEEP above); false when the layout
// does not meet the tensor-copy alignment rules.
bool ct_axis0_stiffness_tma_f32(int n0, bool keep, cplx<float>* X, int64_t P, int64_t cstride,
                                int64_t bstride, int batch, const FusedParams<float>& fp,
                                BatchMask mask, cudaStream_t st);
void ct_set_smem_attrs_tma_f32(size_t max_smem);
// Float-pair instances (passes_ct_df.cu, passes_df_rows.cu, passes_df_c2c.cu):
// the staged and TMA axis-0 forms, rows and axis-1 passes, lengths 64..512.
bool ct_axis0_stiffness_tma_df(int n0, cplx<df64>* X, int64_t P, int64_t cstride,
                               int64_t bstride, int batch, const FusedParams<df64>& fp,
                               BatchMask mask, cudaStream_t st);
void ct_set_smem_attrs_df_axis0(size_t max_smem);
void ct_set_smem_attrs_df_rows(size_t max_smem);
void ct_set_smem_attrs_df_c2c(size_t max_smem);
void ct_set_smem_attrs(size_t max_smem);

}  // namespace bri17gb
