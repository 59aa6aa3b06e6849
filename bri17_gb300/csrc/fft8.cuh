// fft8.cuh -- register-resident Stockham FFT for power-of-two line lengths.
//
// A line of n = 2^e points (8 <= n <= 1024) is held by T = n / 8 threads,
// thread t owning the eight elements t + T q (q = 0..7).  With the
// self-sorting Stockham ordering, a radix-R stage's butterfly j = t + T m
// reads exactly elements t + T (m + r 8/R), i.e. the thread's own eight
// registers, so every stage computes in registers; between stages the
// outputs go through shared memory once (scattered write, barrier, strided
// read of the thread's own positions, barrier).  The last stage's outputs
// land on the thread's own positions in natural order and stay in
// registers: loads and stores of whole lines are coalesced and every thread
// does the same work in every stage.
#pragma once

#include "fft.cuh"

namespace bri17gb {

struct Plan8 {
  int n;        // line length (power of two, 8..1024)
  int T;        // threads per line = n / 8
  int nst;      // stages
  int radix[6]; // 8, 4 or 2
};

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Stage radices: as many 8s as possible, the remainder as 4 x 4 or 4 or 2.
inline bool make_plan8(int n, Plan8* p) {
  if (!is_pow2(n) || n < 8 || n > 1024) return false;
  int e = 0;
  while ((1 << e) < n) e++;
  p->n = n;
  p->T = n / 8;
  p->nst = 0;
  int a = e / 3, b = e % 3;
  if (b == 1) {
    a -= 1;
    for (int i = 0; i < a; i++) p->radix[p->nst++] = 8;
    p->radix[p->nst++] = 4;
    p->radix[p->nst++] = 4;
  } else {
    for (int i = 0; i < a; i++) p->radix[p->nst++] = 8;
    if (b == 2) p->radix[p->nst++] = 4;
  }
  return true;
}

// Shared-memory position of element p of a line: one pad slot per 16.
__device__ __forceinline__ int pad16(int p) { return p + (p >> 4); }
// Position of element p in an exchange buffer: the line's own padded buffer
// (BS = 0), or every BS-th entry (BS > 0: the line interleaved with BS - 1
// others, as in a staged tile laid out [p][line]).
template <int BS>
__device__ __forceinline__ int xpos(int p) {
  return BS > 0 ? p * BS : pad16(p);
}
// Line pitch (complex elements, odd so consecutive lines use distinct banks).
__host__ __device__ __forceinline__ int pitch8(int n) { return n + n / 16 + 1; }

// Pitch (complex elements) of the exchange buffers of `lines` lines of
// length n (a power of two, 8..1024) held by one CTA with the E-element
// engine (8 or 16 elements per thread), for elements of csize bytes.  lines_fastest: consecutive threads
// step across the lines first (thread = t * lines + line, the strided-axis
// passes); otherwise along a line first (thread = line * (n/8) + t, the row
// passes).  Chosen among n + n/16 + {0..15} by a model of the exchanges'
// shared-memory wavefronts (every stage's scattered writes and strided
// reads, 32 banks of 4 bytes); cached per argument set (host, thread-safe).
int exchange_pitch(int n, int lines, int csize, bool lines_fastest, int E = 8);

// Pitch of lines accessed only in natural order with warp lanes stepping
// across the TB lines first: lines stagger by 32 / TB elements modulo the M
// complex elements of a 128-byte bank row, so a warp's 32 lanes use every
// bank the minimum number of times.
__host__ __device__ __forceinline__ int stash_pitch(int n, int TB, int csize) {
  const int M = 128 / csize;
  const int s = TB >= 1 && TB <= 32 ? 32 / TB : 1;
  return (n + M - 1) / M * M + (s % M == 0 ? M / 2 + 1 : s % M);
}

// One radix-R stage with E elements per thread (E/R butterflies per thread);
// BS as in xpos.
template <typename T, int R, int E, bool INV, int BS = 0>
__device__ __forceinline__ void stageE(cplx<T> (&v)[E], cplx<T>* buf, int t, int TT,
                                       int Ns, int n, const cplx<T>* __restrict__ tw,
                                       int tws, bool last) {
  constexpr int M = E / R;
  const int tstep = (n / (Ns * R)) * tws;
#pragma unroll
  for (int m = 0; m < M; m++) {
    const int j = t + TT * m;
    const int jm = j & (Ns - 1);
    cplx<T> a[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = v[m + r * M];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) a[r] = cmul<T>(a[r], twid<T, INV>(tw, jm * r * tstep));
    }
    dft<T, R, INV>(a);
    if (last) {
#pragma unroll
      for (int r = 0; r < R; r++) v[m + r * M] = a[r];
    } else {
      const int d = (j - jm) * R + jm;
#pragma unroll
      for (int r = 0; r < R; r++) buf[xpos<BS>(d + r * Ns)] = a[r];
    }
  }
}

template <typename T, int R, bool INV>
__device__ __forceinline__ void stage8(cplx<T> (&v)[8], cplx<T>* buf, int t, int TT,
                                       int Ns, int n, const cplx<T>* __restrict__ tw,
                                       int tws, bool last) {
  stageE<T, R, 8, INV>(v, buf, t, TT, Ns, n, tw, tws, last);
}

// Transform one line held as v[q] = x[t + T q]; the result replaces v in the
// same ownership.  `buf` is this line's exchange buffer (pitch8(n) entries).
// Every thread of the CTA must call it (it contains barriers).
template <typename T, bool INV>
__device__ __forceinline__ void fft8_line(cplx<T> (&v)[8], cplx<T>* buf, int t,
                                          const Plan8& p, const cplx<T>* __restrict__ tw,
                                          int tws) {
  int Ns = 1;
  for (int s = 0; s < p.nst; s++) {
    const int R = p.radix[s];
    const bool last = s == p.nst - 1;
    if (R == 8)
      stage8<T, 8, INV>(v, buf, t, p.T, Ns, p.n, tw, tws, last);
    else if (R == 4)
      stage8<T, 4, INV>(v, buf, t, p.T, Ns, p.n, tw, tws, last);
    else
      stage8<T, 2, INV>(v, buf, t, p.T, Ns, p.n, tw, tws, last);
    if (!last) {
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 8; q++) v[q] = buf[pad16(t + p.T * q)];
      __syncthreads();
    }
    Ns *= R;
  }
}

}  // namespace bri17gb
