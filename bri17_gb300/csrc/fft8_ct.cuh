// fft8_ct.cuh -- compile-time-length form of the register-resident engine
// (fft8.cuh): the line length N and the elements per thread E (8 or 16 for
// powers of two, 12 for 3 * 2^k) are template parameters, so the stage
// radices, spans, twiddle strides and shared-memory positions fold into
// constants and the stage loop unrolls.  Thread t holds elements
// t + (N/E) q, q < E; with E = 16 most powers of two need one shared-memory
// exchange fewer than with E = 8.
#pragma once

#include "fft8.cuh"

namespace bri17gb {

template <int N, int E>
struct PE {
  static_assert((E == 8 || E == 16) && N >= E && N <= 1024 && (N & (N - 1)) == 0,
                "power of two in [E, 1024], E in {8, 16}");
  static constexpr int kE = E;
  static constexpr int T = N / E;
  static constexpr int log2i(int x) {
    int e = 0;
    while ((1 << e) < x) e++;
    return e;
  }
  static constexpr int LN = log2i(N);
  static constexpr int LE = log2i(E);
  // E = 8: 8s, then 4x4 (LN % 3 == 1) or 4 (LN % 3 == 2).
  // E = 16: 16s, then one stage of the remaining power of two.
  static constexpr int NST =
      E == 8 ? ((LN % 3 == 1) ? (LN / 3 + 1) : (LN / 3 + (LN % 3 == 2 ? 1 : 0)))
             : (LN / 4 + (LN % 4 ? 1 : 0));
  static constexpr int radix(int s) {
    return E == 8 ? ((LN % 3 == 1) ? (s < LN / 3 - 1 ? 8 : 4) : (s < LN / 3 ? 8 : 4))
                  : (s < LN / 4 ? 16 : (1 << (LN % 4)));
  }
  // Product of the radices before stage s.
  static constexpr int ns(int s) {
    int p = 1;
    for (int i = 0; i < s; i++) p *= radix(i);
    return p;
  }
  // Per-stage twiddle table: stage s >= 1 holds W^(jm r tstep) at
  // (r - 1) ns(s) + jm, r in [1, R), jm in [0, ns(s)), after the stages
  // before it; stage 0 has none.  N - radix(0) entries in all.
  static constexpr int twoff(int s) {
    int o = 0;
    for (int i = 1; i < s; i++) o += (radix(i) - 1) * ns(i);
    return o;
  }
  static constexpr int TWN = N - (NST > 0 ? radix(0) : N);
};

// Lengths N = 3 * 2^k, 24 <= N <= 768: twelve elements per thread, radix-4
// stages (one radix-2 stage when k is odd), then one radix-3 stage.  With
// the radix 3 last, every stage before it spans a power of two, so the
// stage code's jm = j mod Ns is a mask as for the power-of-two lengths, and
// every radix divides E (the Stockham butterflies of a thread read only its
// own registers).  Same members as PE.
template <int N>
struct PE3 {
  static constexpr int kE = 12;
  static constexpr int P = N / 3;
  static_assert(N % 3 == 0 && (P & (P - 1)) == 0 && P >= 8 && N <= 768, "3 * 2^k in 24..768");
  static constexpr int T = N / kE;
  static constexpr int LP = PE<16, 16>::log2i(P);
  static constexpr int NST = LP / 2 + LP % 2 + 1;
  static constexpr int radix(int s) { return s == NST - 1 ? 3 : (s < LP / 2 ? 4 : 2); }
  static constexpr int ns(int s) {
    int p = 1;
    for (int i = 0; i < s; i++) p *= radix(i);
    return p;
  }
  static constexpr int twoff(int s) {
    int o = 0;
    for (int i = 1; i < s; i++) o += (radix(i) - 1) * ns(i);
    return o;
  }
  static constexpr int TWN = N - radix(0);
};

// Fills the per-stage twiddle table of schedule P (PE or PE3) from the
// natural table `tw` (W_{N tws}^i at i, read with stride tws); cooperative
// over `nthr` threads.  Stage by stage at compile time, so the index
// arithmetic folds into constants.
template <typename T, class P, int S>
__device__ __forceinline__ void fftP_twiddles_from(cplx<T>* __restrict__ dst,
                                                   const cplx<T>* __restrict__ tw, int tws,
                                                   int tid, int nthr) {
  if constexpr (S < P::NST) {
    constexpr int NS = P::ns(S), R = P::radix(S), OFF = P::twoff(S);
    constexpr int STEP = P::T * P::kE / (NS * R);
    for (int i = tid; i < (R - 1) * NS; i += nthr) {
      const int r = 1 + i / NS, jm = i % NS;
      dst[OFF + i] = tw[jm * r * STEP * tws];
    }
    fftP_twiddles_from<T, P, S + 1>(dst, tw, tws, tid, nthr);
  }
}

template <typename T, class P>
__device__ __forceinline__ void fftP_twiddles(cplx<T>* __restrict__ dst,
                                              const cplx<T>* __restrict__ tw, int tws, int tid,
                                              int nthr) {
  fftP_twiddles_from<T, P, 1>(dst, tw, tws, tid, nthr);
}

template <typename T, int N, int E>
__device__ __forceinline__ void fftE_ct_twiddles(cplx<T>* __restrict__ dst,
                                                 const cplx<T>* __restrict__ tw, int tws,
                                                 int tid, int nthr) {
  fftP_twiddles<T, PE<N, E>>(dst, tw, tws, tid, nthr);
}

// One radix-R stage reading its twiddles from the per-stage table `stw`
// (consecutive butterflies, consecutive entries: no bank conflicts).
template <typename T, int R, int E, bool INV>
__device__ __forceinline__ void stageE_st(cplx<T> (&v)[E], cplx<T>* buf, int t, int TT,
                                          int Ns, const cplx<T>* __restrict__ stw, bool last) {
  constexpr int M = E / R;
#pragma unroll
  for (int m = 0; m < M; m++) {
    const int j = t + TT * m;
    const int jm = j & (Ns - 1);
    cplx<T> a[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = v[m + r * M];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) a[r] = cmul<T>(a[r], twid<T, INV>(stw, (r - 1) * Ns + jm));
    }
    dft<T, R, INV>(a);
    if (last) {
#pragma unroll
      for (int r = 0; r < R; r++) v[m + r * M] = a[r];
    } else {
      const int d = (j - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; r++) buf[pad16(d + r * Ns)] = a[r];
    }
  }
}

// `stw`: the per-stage twiddle table (fftP_twiddles).
template <typename T, class P, bool INV, int S, int NS>
__device__ __forceinline__ void fftP_stage(cplx<T> (&v)[P::kE], cplx<T>* buf, int t,
                                           const cplx<T>* __restrict__ stw) {
  constexpr int R = P::radix(S);
  constexpr bool LAST = S == P::NST - 1;
  stageE_st<T, R, P::kE, INV>(v, buf, t, P::T, NS, stw + (S > 0 ? P::twoff(S) : 0), LAST);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < P::kE; q++) v[q] = buf[pad16(t + P::T * q)];
    __syncthreads();
    fftP_stage<T, P, INV, S + 1, NS * R>(v, buf, t, stw);
  }
}

// Transform one line held as v[q] = x[t + T q] (see fft8_line), T = N / E,
// with the per-stage twiddle table `stw` of schedule P (fftP_twiddles).
template <typename T, class P, bool INV>
__device__ __forceinline__ void fftP(cplx<T> (&v)[P::kE], cplx<T>* buf, int t,
                                     const cplx<T>* __restrict__ stw) {
  fftP_stage<T, P, INV, 0, 1>(v, buf, t, stw);
}

template <typename T, int N, int E, bool INV>
__device__ __forceinline__ void fftE_ct(cplx<T> (&v)[E], cplx<T>* buf, int t,
                                        const cplx<T>* __restrict__ stw) {
  fftP<T, PE<N, E>, INV>(v, buf, t, stw);
}

// The same transform reading the natural table `tw` with stride tws; the
// exchanges go through `buf` at xpos<BS> (BS = 0: the line's own padded
// buffer).
template <typename T, int N, int E, bool INV, int S, int NS, int BS = 0>
__device__ __forceinline__ void fftE_ct_stage_nat(cplx<T> (&v)[E], cplx<T>* buf, int t,
                                                  const cplx<T>* __restrict__ tw, int tws) {
  constexpr int R = PE<N, E>::radix(S);
  constexpr bool LAST = S == PE<N, E>::NST - 1;
  stageE<T, R, E, INV, BS>(v, buf, t, PE<N, E>::T, NS, N, tw, tws, LAST);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = buf[xpos<BS>(t + PE<N, E>::T * q)];
    __syncthreads();
    fftE_ct_stage_nat<T, N, E, INV, S + 1, NS * R, BS>(v, buf, t, tw, tws);
  }
}

template <typename T, int N, int E, bool INV, int BS = 0>
__device__ __forceinline__ void fftE_ct_nat(cplx<T> (&v)[E], cplx<T>* buf, int t,
                                            const cplx<T>* __restrict__ tw, int tws) {
  fftE_ct_stage_nat<T, N, E, INV, 0, 1, BS>(v, buf, t, tw, tws);
}



}  // namespace bri17gb
