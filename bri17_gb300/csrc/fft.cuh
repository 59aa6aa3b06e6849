// fft.cuh -- shared-memory Stockham FFT engine for batches of lines.
//
// Replaces the FFTW3 complex transforms of the reference's operator
// application (fftw_plan_dft / fftw_execute, tests/test_bri17.cpp:57, :95,
// :121-126).  A CTA holds a tile of lines in shared memory and runs
// self-sorting (Stockham, decimation in time) radix stages over it,
// ping-ponging between two buffers.  Hand-written butterflies cover radices
// 2, 3, 4, 5, 8 and 16; any other odd prime radix up to kMaxGenericRadix runs
// through a generic O(r^2) butterfly built on the axis twiddle table.
//
// Convention: forward = sum x[n] exp(-2 pi i n k / N) (sphinx/theory.rst
// eq. (1)); inverse = the unnormalised conjugate transform (FFTW_BACKWARD).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bri17gb {

constexpr int kMaxStages = 12;
constexpr int kMaxGenericRadix = 61;

// Radix sequence of one line length.  n == 1 has no stage.
struct AxisPlan {
  int n;
  int nstages;
  int radix[kMaxStages];
};

template <typename T>
struct CplxOf;
template <>
struct CplxOf<double> {
  using type = double2;
};
template <>
struct CplxOf<float> {
  using type = float2;
};
template <typename T>
using cplx = typename CplxOf<T>::type;

template <typename T>
__device__ __forceinline__ cplx<T> mk(T x, T y) {
  cplx<T> r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename T>
__device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cplx<T> cmulc(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T>
__device__ __forceinline__ cplx<T> cscale(cplx<T> a, T s) {
  return mk<T>(a.x * s, a.y * s);
}
// Multiply by -i (forward) or +i (inverse).
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> rot(cplx<T> a) {
  return INV ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}
// Twiddle W^t (table holds exp(-2 pi i t / n)); conjugated for the inverse.
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> twid(const cplx<T>* tw, int t) {
  cplx<T> w = tw[t];
  if (INV) w.y = -w.y;
  return w;
}
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> tmul(cplx<T> a, T c, T s) {
  // a * (c - i s) forward, a * (c + i s) inverse.
  return INV ? mk<T>(a.x * c - a.y * s, a.x * s + a.y * c)
             : mk<T>(a.x * c + a.y * s, a.y * c - a.x * s);
}

// ---------------------------------------------------------------------------
// Butterflies: in-register DFT of length R, natural order in and out.

template <typename T, bool INV>
__device__ __forceinline__ void dft2(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1];
  v[0] = cadd<T>(a, b);
  v[1] = csub<T>(a, b);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft3(cplx<T>* v) {
  const T kC = T(0.5);
  const T kS = T(0.8660254037844386467637231707529361834714);  // sqrt(3)/2
  cplx<T> t1 = cadd<T>(v[1], v[2]);
  cplx<T> t2 = mk<T>(v[0].x - kC * t1.x, v[0].y - kC * t1.y);
  cplx<T> d = csub<T>(v[1], v[2]);
  cplx<T> t3 = rot<T, INV>(mk<T>(kS * d.x, kS * d.y));
  v[0] = cadd<T>(v[0], t1);
  v[1] = cadd<T>(t2, t3);
  v[2] = csub<T>(t2, t3);
}

// Sums inside a butterfly: cadd / csub, except that float pairs (df64.cuh)
// leave out the renormalisation of each sum; bnorm restores it on values
// that leave the butterfly.  For float and double all three are the plain
// operations.
template <typename T>
__device__ __forceinline__ cplx<T> badd(cplx<T> a, cplx<T> b) {
  return cadd<T>(a, b);
}
template <typename T>
__device__ __forceinline__ cplx<T> bsub(cplx<T> a, cplx<T> b) {
  return csub<T>(a, b);
}
template <typename T>
__device__ __forceinline__ cplx<T> bnorm(cplx<T> a) {
  return a;
}

// NORM = false leaves the outputs unnormalised (for a caller that goes on
// summing them, as dft8 does).
template <typename T, bool INV, bool NORM = true>
__device__ __forceinline__ void dft4(cplx<T>* v) {
  cplx<T> t0 = badd<T>(v[0], v[2]);
  cplx<T> t1 = bsub<T>(v[0], v[2]);
  cplx<T> t2 = badd<T>(v[1], v[3]);
  cplx<T> t3 = rot<T, INV>(bsub<T>(v[1], v[3]));
  if constexpr (NORM) {
    v[0] = bnorm<T>(badd<T>(t0, t2));
    v[2] = bnorm<T>(bsub<T>(t0, t2));
    v[1] = bnorm<T>(badd<T>(t1, t3));
    v[3] = bnorm<T>(bsub<T>(t1, t3));
  } else {
    v[0] = badd<T>(t0, t2);
    v[2] = bsub<T>(t0, t2);
    v[1] = badd<T>(t1, t3);
    v[3] = bsub<T>(t1, t3);
  }
}

template <typename T, bool INV>
__device__ __forceinline__ void dft5(cplx<T>* v) {
  const T c1 = T(0.3090169943749474241022934171828190588602);
  const T c2 = T(-0.8090169943749474241022934171828190588602);
  const T s1 = T(0.9510565162951535721164393333793821434057);
  const T s2 = T(0.5877852522924731291687059546390727685976);
  cplx<T> t1 = cadd<T>(v[1], v[4]);
  cplx<T> t2 = cadd<T>(v[2], v[3]);
  cplx<T> t3 = csub<T>(v[1], v[4]);
  cplx<T> t4 = csub<T>(v[2], v[3]);
  cplx<T> a0 = v[0];
  cplx<T> b1 = mk<T>(a0.x + c1 * t1.x + c2 * t2.x, a0.y + c1 * t1.y + c2 * t2.y);
  cplx<T> b2 = mk<T>(a0.x + c2 * t1.x + c1 * t2.x, a0.y + c2 * t1.y + c1 * t2.y);
  cplx<T> d1 = mk<T>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  cplx<T> d2 = mk<T>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  cplx<T> r1 = rot<T, INV>(d1);  // -i d1 forward
  cplx<T> r2 = rot<T, INV>(d2);
  v[0] = cadd<T>(a0, cadd<T>(t1, t2));
  v[1] = cadd<T>(b1, r1);
  v[4] = csub<T>(b1, r1);
  v[2] = cadd<T>(b2, r2);
  v[3] = csub<T>(b2, r2);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(cplx<T>* v) {
  const T r = T(0.7071067811865475244008443621048490392848);
  cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
  cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T, INV, false>(e);
  dft4<T, INV, false>(o);
  // o[k] *= W8^k
  cplx<T> o1 = INV ? mk<T>(r * (o[1].x - o[1].y), r * (o[1].x + o[1].y))
                   : mk<T>(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x));
  cplx<T> o2 = rot<T, INV>(o[2]);
  cplx<T> o3 = INV ? mk<T>(-r * (o[3].x + o[3].y), r * (o[3].x - o[3].y))
                   : mk<T>(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y));
  v[0] = cadd<T>(e[0], o[0]);
  v[4] = csub<T>(e[0], o[0]);
  v[1] = cadd<T>(e[1], o1);
  v[5] = csub<T>(e[1], o1);
  v[2] = cadd<T>(e[2], o2);
  v[6] = csub<T>(e[2], o2);
  v[3] = cadd<T>(e[3], o3);
  v[7] = csub<T>(e[3], o3);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft16(cplx<T>* v) {
  // 16 = 4 x 4: inner DFT4 over n2 (stride 4), twiddle W16^(n1 k2), outer
  // DFT4 over n1; X[k2 + 4 k1].
  const T c1 = T(0.9238795325112867561281831893967882868224);  // cos(pi/8)
  const T s1 = T(0.3826834323650897717284599840303988667613);  // sin(pi/8)
  const T r = T(0.7071067811865475244008443621048490392848);
  cplx<T> b[4][4];
#pragma unroll
  for (int n1 = 0; n1 < 4; n1++) {
    cplx<T> col[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
    dft4<T, INV>(col);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) b[n1][k2] = col[k2];
  }
  // W16^j for j = n1*k2 in {1,2,3,4,6,9}.
  b[1][1] = tmul<T, INV>(b[1][1], c1, s1);
  b[1][2] = tmul<T, INV>(b[1][2], r, r);
  b[1][3] = tmul<T, INV>(b[1][3], s1, c1);
  b[2][1] = tmul<T, INV>(b[2][1], r, r);
  b[2][2] = rot<T, INV>(b[2][2]);
  b[2][3] = tmul<T, INV>(b[2][3], -r, r);
  b[3][1] = tmul<T, INV>(b[3][1], s1, c1);
  b[3][2] = tmul<T, INV>(b[3][2], -r, r);
  b[3][3] = tmul<T, INV>(b[3][3], -c1, -s1);
#pragma unroll
  for (int k2 = 0; k2 < 4; k2++) {
    cplx<T> row[4] = {b[0][k2], b[1][k2], b[2][k2], b[3][k2]};
    dft4<T, INV>(row);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) v[k2 + 4 * k1] = row[k1];
  }
}

template <typename T, int R, bool INV>
__device__ __forceinline__ void dft(cplx<T>* v) {
  if constexpr (R == 2) dft2<T, INV>(v);
  if constexpr (R == 3) dft3<T, INV>(v);
  if constexpr (R == 4) dft4<T, INV>(v);
  if constexpr (R == 5) dft5<T, INV>(v);
  if constexpr (R == 8) dft8<T, INV>(v);
  if constexpr (R == 16) dft16<T, INV>(v);
}

// ---------------------------------------------------------------------------
// One Stockham stage over `nlines` lines of length n (line pitch `pitch`).
// Ns = product of the radices already applied.  The twiddle table `tw`
// holds exp(-2 pi i t / (n * tws)) at index t; W_n^t is tw[t * tws].

template <typename T, int R, bool INV>
__device__ __forceinline__ void stockham_stage(const cplx<T>* __restrict__ in,
                                               cplx<T>* __restrict__ out,
                                               int nlines, int n, int pitch,
                                               int Ns, const cplx<T>* tw,
                                               int tws) {
  const int nb = n / R;
  const int total = nb * nlines;
  const int twstep = (n / (Ns * R)) * tws;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int line = t / nb;
    const int j = t - line * nb;
    const cplx<T>* src = in + line * pitch;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * nb];
    const int jm = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++)
        v[r] = cmul<T>(v[r], twid<T, INV>(tw, jm * r * twstep));
    }
    dft<T, R, INV>(v);
    const int d = (j - jm) * R + jm;
    cplx<T>* dst = out + line * pitch;
#pragma unroll
    for (int r = 0; r < R; r++) dst[d + r * Ns] = v[r];
  }
}

// Generic odd radix: z_p = sum_q y_q W_R^(p q), with W_R = W_n^(n/R).
template <typename T, bool INV>
__device__ void stockham_stage_generic(const cplx<T>* __restrict__ in,
                                       cplx<T>* __restrict__ out, int nlines,
                                       int n, int pitch, int Ns, int R,
                                       const cplx<T>* tw, int tws) {
  const int nb = n / R;
  const int total = nb * nlines;
  const int twstep = (n / (Ns * R)) * tws;
  const int rstep = nb * tws;  // W_R^1 = W_n^(n/R)
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int line = t / nb;
    const int j = t - line * nb;
    const cplx<T>* src = in + line * pitch;
    const int jm = j % Ns;
    const int d = (j - jm) * R + jm;
    cplx<T>* dst = out + line * pitch;
    for (int p = 0; p < R; p++) {
      cplx<T> acc = mk<T>(T(0), T(0));
      for (int q = 0; q < R; q++) {
        cplx<T> y = src[j + q * nb];
        if (Ns > 1 && q > 0) y = cmul<T>(y, twid<T, INV>(tw, jm * q * twstep));
        const int e = (p * q) % R;
        acc = cadd<T>(acc, e == 0 ? y : cmul<T>(y, twid<T, INV>(tw, e * rstep)));
      }
      dst[d + p * Ns] = acc;
    }
  }
}

// Transform `nlines` lines held in `a` (pitch `pitch`), using `b` as the
// ping-pong buffer.  The result ends in `a`.  Must be called by every thread
// of the CTA; begins and ends with a barrier-consistent state.
template <typename T, bool INV>
__device__ void fft_lines(cplx<T>* a, cplx<T>* b, int nlines, int pitch,
                          const AxisPlan& p, const cplx<T>* tw, int tws) {
  cplx<T>* src = a;
  cplx<T>* dst = b;
  int Ns = 1;
  for (int s = 0; s < p.nstages; s++) {
    const int R = p.radix[s];
    switch (R) {
      case 2: stockham_stage<T, 2, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      case 3: stockham_stage<T, 3, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      case 4: stockham_stage<T, 4, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      case 5: stockham_stage<T, 5, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      case 8: stockham_stage<T, 8, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      case 16: stockham_stage<T, 16, INV>(src, dst, nlines, p.n, pitch, Ns, tw, tws); break;
      default:
        stockham_stage_generic<T, INV>(src, dst, nlines, p.n, pitch, Ns, R, tw, tws);
        break;
    }
    __syncthreads();
    Ns *= R;
    cplx<T>* tmp = src;
    src = dst;
    dst = tmp;
  }
  if (src != a) {
    const int total = nlines * p.n;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int line = t / p.n;
      const int i = t - line * p.n;
      a[line * pitch + i] = src[line * pitch + i];
    }
    __syncthreads();
  }
}

}  // namespace bri17gb
