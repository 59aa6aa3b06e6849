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
