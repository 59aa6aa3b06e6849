// reduce.cuh -- CG state and deterministic block reductions shared by the
// solver (cg.cu) and the server (server.cu).
#pragma once

#include "op.cuh"

namespace bri17gb {

constexpr int kRedThreads = 256;
constexpr int kRedMaxBlocks = 1024;
constexpr int kChunk = 8;  // CG iterations per graph replay

struct CgState {
  double rr;      // r.r of the current iterate
  double pq;      // p.K p
  double alpha;
  double beta;
  double thresh;  // stop when rr <= thresh
  double aux;     // scratch result of helper reductions
  double mean[6]; // per-component means (projection)
  double rmax2;   // reliable updates: squared FP64 residual at the last update
  int active;     // 1 while iterating
  int pause;      // set by the update kernel: stop after this iteration's
                  // search-direction update (k_apply_pause)
  int flag;       // BRI17_OK or BRI17_ERR_BREAKDOWN
  int iters;
  unsigned int counter;  // last-block ticket
};

inline int red_blocks(int64_t n) {
  int64_t b = (n + kRedThreads * 4 - 1) / (kRedThreads * 4);
  if (b < 1) b = 1;
  if (b > kRedMaxBlocks) b = kRedMaxBlocks;
  return (int)b;
}

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = l < kRedThreads / 32 ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

// Writes this block's partial; returns true in every thread of the last
// block to finish, with *total = fixed-order sum of all partials.
__device__ __forceinline__ bool last_block_total(double v, double* partials,
                                 unsigned int* counter, int nparts,
                                 double* total) {
  __shared__ bool is_last;
  const double b = block_sum(v);
  if (threadIdx.x == 0) {
    partials[blockIdx.x + blockIdx.y * gridDim.x] = b;
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == (unsigned int)nparts - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x)
    s += __ldcg(partials + i);
  const double tot = block_sum(s);
  if (threadIdx.x == 0) {
    *total = tot;
    *counter = 0u;
  }
  return true;
}


// 16-byte vectors of the CG streams: float4 / double2.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int W = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int W = 2;
};
template <typename T>
__device__ __forceinline__ T vget(const typename Vec16<T>::type& v, int i) {
  return reinterpret_cast<const T*>(&v)[i];
}
template <typename T>
__device__ __forceinline__ void vset(typename Vec16<T>::type& v, int i, T x) {
  reinterpret_cast<T*>(&v)[i] = x;
}

// The CG vector kernels below stream their operands as 16-byte vectors, two
// per thread per trip (several independent loads in flight per thread), and
// finish the n mod W tail element-wise.  n is the length of one vector.
// Operands that are not all 16-byte aligned (slot offsets of odd-sized grids
// in a batch) take the element-wise loop for everything.
__device__ __forceinline__ bool aligned16(const void* a, const void* b, const void* c = nullptr,
                                          const void* d = nullptr) {
  return ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
           reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(d)) &
          15u) == 0;
}

// Per-thread accumulator type of the vector reductions: a thread sums its
// share (a few dozen terms) in the vectors' own precision and hands one
// partial to the FP64 block/grid reduction.  FP32 streams thus never touch
// the FP64 pipe per element (on GB300 it runs at 1/64 of the FP32 rate:
// converting and accumulating every element in FP64 made a 50 M-element dot
// product FP64-bound at 4x the time of the memory traffic).
template <typename T>
using Acc = T;

// sum p.q of one vector.
template <typename T>
__device__ __forceinline__ double vdot(const T* __restrict__ p, const T* __restrict__ q,
                                       int64_t n, int64_t tid, int64_t nthreads) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  const int64_t nv = aligned16(p, q) ? n / W : 0;
  const V* pv = reinterpret_cast<const V*>(p);
  const V* qv = reinterpret_cast<const V*>(q);
  Acc<T> a0[W], a1[W];
#pragma unroll
  for (int k = 0; k < W; k++) a0[k] = a1[k] = Acc<T>(0);
  int64_t i = tid;
  for (; i + nthreads < nv; i += 2 * nthreads) {
    const V p0 = pv[i], q0 = qv[i], p1 = pv[i + nthreads], q1 = qv[i + nthreads];
#pragma unroll
    for (int k = 0; k < W; k++) {
      a0[k] += vget<T>(p0, k) * vget<T>(q0, k);
      a1[k] += vget<T>(p1, k) * vget<T>(q1, k);
    }
  }
  for (; i < nv; i += nthreads) {
    const V p0 = pv[i], q0 = qv[i];
#pragma unroll
    for (int k = 0; k < W; k++) a0[k] += vget<T>(p0, k) * vget<T>(q0, k);
  }
  double tot = 0.0;
#pragma unroll
  for (int k = 0; k < W; k++) tot += (double)a0[k] + (double)a1[k];
  for (int64_t j = nv * W + tid; j < n; j += nthreads) tot += (double)p[j] * (double)q[j];
  return tot;
}

// x += a p; r -= a q; returns sum r.r.
template <typename T>
__device__ __forceinline__ double vupdate(T* __restrict__ x, T* __restrict__ r,
                                          const T* __restrict__ p, const T* __restrict__ q,
                                          T a, int64_t n, int64_t tid, int64_t nthreads) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  const int64_t nv = aligned16(x, r, p, q) ? n / W : 0;
  V* xv = reinterpret_cast<V*>(x);
  V* rv = reinterpret_cast<V*>(r);
  const V* pv = reinterpret_cast<const V*>(p);
  const V* qv = reinterpret_cast<const V*>(q);
  Acc<T> acc[W];
#pragma unroll
  for (int k = 0; k < W; k++) acc[k] = Acc<T>(0);
  for (int64_t i = tid; i < nv; i += nthreads) {
    V xi = xv[i], ri = rv[i];
    const V pi = pv[i], qi = qv[i];
#pragma unroll
    for (int k = 0; k < W; k++) {
      vset<T>(xi, k, vget<T>(xi, k) + a * vget<T>(pi, k));
      const T rk = vget<T>(ri, k) - a * vget<T>(qi, k);
      vset<T>(ri, k, rk);
      acc[k] += rk * rk;
    }
    xv[i] = xi;
    rv[i] = ri;
  }
  double tot = 0.0;
#pragma unroll
  for (int k = 0; k < W; k++) tot += (double)acc[k];
  for (int64_t j = nv * W + tid; j < n; j += nthreads) {
    x[j] += a * p[j];
    const T rk = r[j] - a * q[j];
    r[j] = rk;
    tot += (double)rk * (double)rk;
  }
  return tot;
}

// p = r + b p.
template <typename T>
__device__ __forceinline__ void vpupdate(T* __restrict__ p, const T* __restrict__ r, T b,
                                         int64_t n, int64_t tid, int64_t nthreads) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  const int64_t nv = aligned16(p, r) ? n / W : 0;
  V* pv = reinterpret_cast<V*>(p);
  const V* rv = reinterpret_cast<const V*>(r);
  int64_t i = tid;
  for (; i + nthreads < nv; i += 2 * nthreads) {
    V p0 = pv[i], p1 = pv[i + nthreads];
    const V r0 = rv[i], r1 = rv[i + nthreads];
#pragma unroll
    for (int k = 0; k < W; k++) {
      vset<T>(p0, k, vget<T>(r0, k) + b * vget<T>(p0, k));
      vset<T>(p1, k, vget<T>(r1, k) + b * vget<T>(p1, k));
    }
    pv[i] = p0;
    pv[i + nthreads] = p1;
  }
  for (; i < nv; i += nthreads) {
    V p0 = pv[i];
    const V r0 = rv[i];
#pragma unroll
    for (int k = 0; k < W; k++) vset<T>(p0, k, vget<T>(r0, k) + b * vget<T>(p0, k));
    pv[i] = p0;
  }
  for (int64_t j = nv * W + tid; j < n; j += nthreads) p[j] = r[j] + b * p[j];
}

// Ends iteration for states whose update kernel asked to pause: runs after
// the search-direction update, so a paused CG resumes with a consistent p.
static __global__ void k_apply_pause(CgState* sts, int count) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z < count && sts[z].pause) {
    sts[z].active = 0;
    sts[z].pause = 0;
  }
}

}  // namespace bri17gb
