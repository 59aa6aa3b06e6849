// cgstate.cuh -- the conjugate-gradient state and the deterministic block
// reductions, shared by the vector kernels (reduce.cuh), the solver and
// server, and the operator passes that carry a CG reduction (passes_p2.cuh).
#pragma once

#include <stdint.h>

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


// Sum over a CTA of any size (not necessarily a multiple of 32, at most
// 1024 threads) in a fixed order; the result is valid in thread 0.  Every
// thread of the CTA must call it.
__device__ __forceinline__ double block_sum_any(double v) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = ((int)blockDim.x + 31) >> 5;
  const int nl = min(32, (int)blockDim.x - warp * 32);  // lanes of this warp
  const unsigned int m = nl == 32 ? 0xffffffffu : ((1u << nl) - 1u);
  for (int o = 16; o > 0; o >>= 1) {
    const double x = __shfl_down_sync(m, v, o);
    if (lane + o < nl) v += x;
  }
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    const int nl0 = min(32, (int)blockDim.x);
    const unsigned int m0 = nl0 == 32 ? 0xffffffffu : ((1u << nl0) - 1u);
    t = lane < nw ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      const double x = __shfl_down_sync(m0, t, o);
      if (lane + o < nl0) t += x;
    }
  }
  return t;
}

// last_block_total for a reduction carried by an operator pass: this CTA's
// partial goes to partials[base + blockIdx.x]; the ticket counts CTAs over
// all launches of the reduction, and the CTA that takes ticket nparts - 1
// sums all nparts partials in a fixed order.  Every thread of the CTA must
// call it.
__device__ __forceinline__ bool last_block_total_at(double v, double* partials,
                                                    unsigned int* counter, int64_t base,
                                                    int64_t nparts, double* total) {
  __shared__ bool is_last;
  const double b = block_sum_any(v);
  if (threadIdx.x == 0) {
    partials[base + blockIdx.x] = b;
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == (unsigned int)(nparts - 1));
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < nparts; i += blockDim.x) s += __ldcg(partials + i);
  const double tot = block_sum_any(s);
  if (threadIdx.x == 0) {
    *total = tot;
    *counter = 0u;
  }
  return true;
}

}  // namespace bri17gb
