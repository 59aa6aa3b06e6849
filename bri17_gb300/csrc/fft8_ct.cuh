// fft8_ct.cuh -- compile-time-length form of the register-resident engine
// (fft8.cuh): the line length N and the elements per thread E (8 or 16) are
// template parameters, so the stage radices, spans, twiddle strides and
// shared-memory positions fold into constants and the stage loop unrolls.
// Thread t holds elements t + (N/E) q, q < E; with E = 16 most lengths need
// one shared-memory exchange fewer than with E = 8.
#pragma once

#include "fft8.cuh"

namespace bri17gb {

template <int N, int E>
struct PE {
  static_assert((E == 8 || E == 16) && N >= E && N <= 1024 && (N & (N - 1)) == 0,
                "power of two in [E, 1024], E in {8, 16}");
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
};

template <typename T, int N, int E, bool INV, int S, int NS>
__device__ __forceinline__ void fftE_ct_stage(cplx<T> (&v)[E], cplx<T>* buf, int t,
                                              const cplx<T>* __restrict__ tw, int tws) {
  constexpr int R = PE<N, E>::radix(S);
  constexpr bool LAST = S == PE<N, E>::NST - 1;
  stageE<T, R, E, INV>(v, buf, t, PE<N, E>::T, NS, N, tw, tws, LAST);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E; q++) v[q] = buf[pad16(t + PE<N, E>::T * q)];
    __syncthreads();
    fftE_ct_stage<T, N, E, INV, S + 1, NS * R>(v, buf, t, tw, tws);
  }
}

// Transform one line held as v[q] = x[t + (N/E) q] (see fft8_line).
template <typename T, int N, int E, bool INV>
__device__ __forceinline__ void fftE_ct(cplx<T> (&v)[E], cplx<T>* buf, int t,
                                        const cplx<T>* __restrict__ tw, int tws) {
  fftE_ct_stage<T, N, E, INV, 0, 1>(v, buf, t, tw, tws);
}

template <typename T, int N, bool INV>
__device__ __forceinline__ void fft8_ct(cplx<T> (&v)[8], cplx<T>* buf, int t,
                                        const cplx<T>* __restrict__ tw, int tws) {
  fftE_ct<T, N, 8, INV>(v, buf, t, tw, tws);
}

}  // namespace bri17gb
