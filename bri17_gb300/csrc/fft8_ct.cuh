// fft8_ct.cuh -- compile-time-length form of the register-resident engine
// (fft8.cuh): the line length N is a template parameter, so the stage
// radices, spans, twiddle strides and shared-memory positions fold into
// constants and the stage loop unrolls.  Same ownership (thread t holds
// elements t + (N/8) q) and the same results as fft8_line.
#pragma once

#include "fft8.cuh"

namespace bri17gb {

template <int N>
struct P8 {
  static_assert(N >= 8 && N <= 1024 && (N & (N - 1)) == 0, "power of two in [8, 1024]");
  static constexpr int T = N / 8;
  static constexpr int log2n() {
    int e = 0;
    while ((1 << e) < N) e++;
    return e;
  }
  static constexpr int E = log2n();
  // Radices: 8s, then 4x4 (e % 3 == 1) or 4 (e % 3 == 2).
  static constexpr int NST = (E % 3 == 1) ? (E / 3 + 1) : (E / 3 + (E % 3 == 2 ? 1 : 0));
  static constexpr int radix(int s) {
    return (E % 3 == 1) ? (s < E / 3 - 1 ? 8 : 4) : (s < E / 3 ? 8 : 4);
  }
};

template <typename T, int N, bool INV, int S, int NS>
__device__ __forceinline__ void fft8_ct_stage(cplx<T> (&v)[8], cplx<T>* buf, int t,
                                              const cplx<T>* __restrict__ tw, int tws) {
  constexpr int R = P8<N>::radix(S);
  constexpr bool LAST = S == P8<N>::NST - 1;
  stage8<T, R, INV>(v, buf, t, P8<N>::T, NS, N, tw, tws, LAST);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = buf[pad16(t + P8<N>::T * q)];
    __syncthreads();
    fft8_ct_stage<T, N, INV, S + 1, NS * R>(v, buf, t, tw, tws);
  }
}

// Transform one line held as v[q] = x[t + (N/8) q] (see fft8_line).
template <typename T, int N, bool INV>
__device__ __forceinline__ void fft8_ct(cplx<T> (&v)[8], cplx<T>* buf, int t,
                                        const cplx<T>* __restrict__ tw, int tws) {
  fft8_ct_stage<T, N, INV, 0, 1>(v, buf, t, tw, tws);
}

}  // namespace bri17gb
