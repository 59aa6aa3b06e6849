// cg.cu -- conjugate-gradient solvers of K x = b on the periodic stiffness
// operator (new: the reference stops at the per-mode solve
// Hooke::modal_eigenstress_to_opposite_strain, include/bri17/bri17.hpp:
// 308-355, which serves as the exact oracle of these solves).
//
// Plain mode runs CG in the handle's precision.  Mixed mode runs an FP32 CG
// on the FP32 twin of the operator inside an FP64 iterative-refinement loop:
// residual r = b - K x, zero-mean projection and the correction x += d are
// FP64.  Scalars (rr, pq, alpha, beta) stay on the device, reductions are
// deterministic (per-block partials summed in a fixed order by the last
// block), and a chunk of iterations is replayed as one CUDA graph between
// host checks of the residual.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "op.cuh"
#include "reduce.cuh"

namespace bri17gb {

// pq = p . q; alpha = rr / pq; breakdown if pq <= 0 or not finite.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_dot_pq(const T* __restrict__ p, const T* __restrict__ q, int64_t n,
             CgState* st, double* partials) {
  if (!st->active) return;
  const double v = vdot<T>(p, q, n, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                           (int64_t)gridDim.x * blockDim.x);
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) &&
      threadIdx.x == 0) {
    st->pq = tot;
    if (!(tot > 0.0) || !isfinite(tot)) {
      st->flag = BRI17_ERR_BREAKDOWN;
      st->active = 0;
    } else {
      st->alpha = st->rr / tot;
    }
  }
}

// x += alpha p; r -= alpha q; rr_new = r.r; beta = rr_new / rr.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_update(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
             const T* __restrict__ q, int64_t n, CgState* st,
             double* partials) {
  if (!st->active) return;
  const double v = vupdate<T>(x, r, p, q, (T)st->alpha, n,
                              (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                              (int64_t)gridDim.x * blockDim.x);
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) &&
      threadIdx.x == 0) {
    st->iters += 1;
    if (!isfinite(tot)) {
      st->flag = BRI17_ERR_BREAKDOWN;
      st->active = 0;
      return;
    }
    st->beta = tot / st->rr;
    st->rr = tot;
    if (tot <= st->thresh) st->pause = 1;
  }
}

// p = r + beta p.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_pupdate(T* __restrict__ p, const T* __restrict__ r, int64_t n,
              const CgState* st) {
  if (!st->active) return;
  vpupdate<T>(p, r, (T)st->beta, n, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
              (int64_t)gridDim.x * blockDim.x);
}

// aux = a . b
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_dot(const T* __restrict__ a, const T* __restrict__ b, int64_t n,
          CgState* st, double* partials) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v += (double)a[i] * (double)b[i];
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) &&
      threadIdx.x == 0)
    st->aux = tot;
}

// aux = |b - kx|^2 (the true residual's square norm, from K x in kx).
__global__ void __launch_bounds__(kRedThreads)
    k_resnorm(const double* __restrict__ b, const double* __restrict__ kx, int64_t n,
              CgState* st, double* partials) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double d = b[i] - kx[i];
    v += d * d;
  }
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) && threadIdx.x == 0)
    st->aux = tot;
}

// Per-component means of a dim x size field (grid.y = component).
__global__ void __launch_bounds__(kRedThreads)
    k_comp_mean(const double* __restrict__ a, int64_t size, CgState* st,
                double* partials) {
  const double* ac = a + (int64_t)blockIdx.y * size;
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size;
       i += (int64_t)gridDim.x * blockDim.x)
    v += ac[i];
  // The per-component sums are finished by the last block over all
  // components, in a fixed order.
  __shared__ bool is_last;
  const double b = block_sum(v);
  const int nparts = gridDim.x * gridDim.y;
  if (threadIdx.x == 0) {
    partials[blockIdx.x + blockIdx.y * gridDim.x] = b;
    __threadfence();
    const unsigned int t = atomicAdd(&st->counter, 1u);
    is_last = (t == (unsigned int)nparts - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int c = 0; c < (int)gridDim.y; c++) {
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
      s += __ldcg(partials + c * gridDim.x + i);
    const double tot = block_sum(s);
    if (threadIdx.x == 0) st->mean[c] = tot / (double)size;
  }
  if (threadIdx.x == 0) st->counter = 0u;
}

__global__ void k_sub_mean(double* __restrict__ a, int64_t size,
                           const CgState* st) {
  const double m = st->mean[blockIdx.y];
  double* ac = a + (int64_t)blockIdx.y * size;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size;
       i += (int64_t)gridDim.x * blockDim.x)
    ac[i] -= m;
}

// r = b - Kx (Kx given), FP64.
__global__ void k_residual(double* __restrict__ r, const double* __restrict__ b,
                           const double* __restrict__ kx, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - kx[i];
}

// out32 = (float)(in64 * scale); zero the FP32 iterate.
__global__ void k_to_f32(float* __restrict__ out, const double* __restrict__ in,
                         double scale, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)(in[i] * scale);
}

// aux = sum (a64 s - b32 t)^2: the squared gap between the recomputed FP64
// residual and the recursive FP32 one, both in the same (scaled) units.
__global__ void __launch_bounds__(kRedThreads)
    k_gap(const double* __restrict__ a, const float* __restrict__ b, double s, double t,
          int64_t n, CgState* st, double* partials) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double g = a[i] * s - (double)b[i] * t;
    v += g * g;
  }
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) && threadIdx.x == 0)
    st->aux = tot;
}

// a32 *= f.
__global__ void k_scale_f32(float* __restrict__ a, float f, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] *= f;
}

// x64 += scale * d32.
__global__ void k_add_f32(double* __restrict__ x, const float* __restrict__ d,
                          double scale, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += scale * (double)d[i];
}

// CG start: p = r; rr = r.r; thresh = rel_tol2 * aux (aux = b.b set by a
// preceding k_dot); active while rr > thresh.
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_start(const T* __restrict__ r, T* __restrict__ p, int64_t n, CgState* st,
            double* partials, double rel_tol2) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T ri = r[i];
    p[i] = ri;
    v += (double)ri * (double)ri;
  }
  double tot;
  if (last_block_total(v, partials, &st->counter, gridDim.x, &tot) &&
      threadIdx.x == 0) {
    st->rr = tot;
    st->thresh = rel_tol2 * st->aux;
    st->iters = 0;
    st->pause = 0;
    st->flag = isfinite(tot) ? BRI17_OK : BRI17_ERR_BREAKDOWN;
    st->active = (tot > st->thresh && isfinite(tot)) ? 1 : 0;
  }
}

// Reliable update: the recursive FP32 residual was just replaced by the
// FP64 one (aux = its squared norm); keep the search direction, resume.
// At least one more chunk runs even when the replaced residual already meets
// the FP32 threshold, so every update changes the iterate.
// The plain solver's resumption after a true-residual check: same CG, a new
// pause threshold.
__global__ void k_plain_resume(CgState* st, double thresh) {
  st->thresh = thresh;
  st->pause = 0;
  st->active = (st->rr > thresh && isfinite(st->rr)) ? 1 : 0;
}

__global__ void k_reliable_resume(CgState* st, double thresh) {
  st->rr = st->aux;
  st->thresh = thresh;
  st->flag = BRI17_OK;
  st->pause = 0;
  st->active = isfinite(st->aux) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Host side.

struct CgWork {
  int64_t n;        // dim * size
  double* x;        // FP64 iterate (work copy)
  double* r;        // FP64 residual
  double* p;        // FP64 search direction (plain mode)
  double* xbest;    // plain mode: the iterate with the smallest true residual seen
  double* q;        // FP64 K p / K x
  float* d32;       // FP32 inner iterate (mixed mode)
  float* r32;
  float* p32;
  float* q32;
  double* partials;
  double* pq_part;   // per-CTA partials of p.Kp from the FP32 stiffness pass
  CgState* st;
  CgState* st_host;  // pinned mirror
  cudaStream_t stream;
  cudaGraphExec_t graph64;
  cudaGraphExec_t graph32;
  unsigned epoch64;
  unsigned epoch32;
  bool plain_ready;
};

static void cg_free(void* p) {
  CgWork* w = reinterpret_cast<CgWork*>(p);
  if (!w) return;
  if (w->stream) cudaStreamSynchronize(w->stream);
  if (w->graph64) cudaGraphExecDestroy(w->graph64);
  if (w->graph32) cudaGraphExecDestroy(w->graph32);
  cudaFree(w->x);
  cudaFree(w->r);
  cudaFree(w->p);
  cudaFree(w->xbest);
  cudaFree(w->q);
  cudaFree(w->d32);
  cudaFree(w->r32);
  cudaFree(w->p32);
  cudaFree(w->q32);
  cudaFree(w->partials);
  cudaFree(w->pq_part);
  cudaFree(w->st);
  cudaFreeHost(w->st_host);
  if (w->stream) cudaStreamDestroy(w->stream);
  delete w;
}

static int ensure_work(bri17_op* op, bool mixed, CgWork** out) {
  CgWork* w = reinterpret_cast<CgWork*>(op->cg_work);
  const int64_t n = (int64_t)op->g.dim * op->g.size;
  if (!w) {
    w = new CgWork();
    memset(w, 0, sizeof(*w));
    w->n = n;
    op->cg_work = w;
    op->cg_free = cg_free;
    BRI17_CUDA_TRY(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    BRI17_CUDA_TRY(cudaMalloc(&w->x, n * sizeof(double)));
    BRI17_CUDA_TRY(cudaMalloc(&w->r, n * sizeof(double)));
    BRI17_CUDA_TRY(cudaMalloc(&w->q, n * sizeof(double)));
    BRI17_CUDA_TRY(cudaMalloc(&w->partials, 6 * kRedMaxBlocks * sizeof(double)));
    BRI17_CUDA_TRY(cudaMalloc(&w->pq_part, (size_t)std::max<int64_t>(op->g.P, 1) * sizeof(double)));
    BRI17_CUDA_TRY(cudaMalloc(&w->st, sizeof(CgState)));
    BRI17_CUDA_TRY(cudaMemset(w->st, 0, sizeof(CgState)));
    BRI17_CUDA_TRY(cudaMallocHost(&w->st_host, sizeof(CgState)));
    memset(w->st_host, 0, sizeof(CgState));
  }
  if (!mixed && !w->plain_ready) {
    if (op->precision == BRI17_F64) {
      BRI17_CUDA_TRY(cudaMalloc(&w->p, n * sizeof(double)));
      BRI17_CUDA_TRY(cudaMalloc(&w->xbest, n * sizeof(double)));
    } else {
      BRI17_CUDA_TRY(cudaMalloc(&w->d32, n * sizeof(float)));
      BRI17_CUDA_TRY(cudaMalloc(&w->r32, n * sizeof(float)));
      BRI17_CUDA_TRY(cudaMalloc(&w->p32, n * sizeof(float)));
      BRI17_CUDA_TRY(cudaMalloc(&w->q32, n * sizeof(float)));
    }
    w->plain_ready = true;
  }
  if (mixed && !w->d32) {  // (an FP32 handle's plain mode allocated these)
    BRI17_CUDA_TRY(cudaMalloc(&w->d32, n * sizeof(float)));
    BRI17_CUDA_TRY(cudaMalloc(&w->r32, n * sizeof(float)));
    BRI17_CUDA_TRY(cudaMalloc(&w->p32, n * sizeof(float)));
    BRI17_CUDA_TRY(cudaMalloc(&w->q32, n * sizeof(float)));
  }
  *out = w;
  return BRI17_OK;
}

static unsigned grid1(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// Enqueue `chunk` CG iterations of precision T on `opk` (the operator whose
// precision is T), then a copy of the state to the pinned mirror.
template <typename T>
static int enqueue_chunk(bri17_op* opk, CgWork* w, T* x, T* r, T* p, T* q,
                         cudaStream_t s) {
  const int64_t n = w->n;
  const int rb = red_blocks(n);
  // FP32: p.Kp summed by Parseval in the stiffness pass where the handle's
  // form allows (no separate pass over p and q).
  bool fused = false;
  if constexpr (std::is_same<T, float>::value) fused = cg_pq_fusable(opk) && w->pq_part;
  for (int it = 0; it < kChunk; it++) {
    int rc;
    if constexpr (std::is_same<T, float>::value) {
      rc = fused ? apply_stiffness_cg_async(opk, p, q, w->st, w->pq_part, s)
                 : apply_stiffness_async(opk, p, q, s);
    } else {
      rc = apply_stiffness_async(opk, p, q, s);
    }
    if (rc != BRI17_OK) return rc;
    if (!fused) k_dot_pq<T><<<rb, kRedThreads, 0, s>>>(p, q, n, w->st, w->partials);
    k_update<T><<<rb, kRedThreads, 0, s>>>(x, r, p, q, n, w->st, w->partials);
    k_pupdate<T><<<grid1(n), 256, 0, s>>>(p, r, n, w->st);
    k_apply_pause<<<1, 32, 0, s>>>(w->st, 1);
  }
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->st_host, w->st, sizeof(CgState),
                                 cudaMemcpyDeviceToHost, s));
  return BRI17_OK;
}

template <typename T>
static int get_graph(bri17_op* opk, CgWork* w, T* x, T* r, T* p, T* q,
                     cudaGraphExec_t* exec, unsigned* epoch) {
  if (*exec && *epoch == opk->material_epoch) return BRI17_OK;
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaGraph_t graph;
  BRI17_CUDA_TRY(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_chunk<T>(opk, w, x, r, p, q, w->stream);
  cudaError_t e = cudaStreamEndCapture(w->stream, &graph);
  if (rc != BRI17_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  *epoch = opk->material_epoch;
  return BRI17_OK;
}

// Run CG iterations (state already started) until inactive or `budget`
// iterations; returns the status flag.  *iters receives the count.
template <typename T>
static int run_cg(bri17_op* opk, CgWork* w, T* x, T* r, T* p, T* q,
                  cudaGraphExec_t* exec, unsigned* epoch, int budget,
                  int* iters) {
  int rc = get_graph<T>(opk, w, x, r, p, q, exec, epoch);
  if (rc != BRI17_OK) return rc;
  // The state was started on w->stream; refresh the mirror first.
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->st_host, w->st, sizeof(CgState),
                                 cudaMemcpyDeviceToHost, w->stream));
  BRI17_CUDA_TRY(cudaStreamSynchronize(w->stream));
  while (w->st_host->active && w->st_host->iters < budget) {
    BRI17_CUDA_TRY(cudaGraphLaunch(*exec, w->stream));
    BRI17_CUDA_TRY(cudaStreamSynchronize(w->stream));
    const int ts = take_status(opk);  // a bounded device wait of the chunk ran out
    if (ts != BRI17_OK) {
      *iters = w->st_host->iters;
      return ts;
    }
  }
  *iters = w->st_host->iters;
  if (w->st_host->flag != BRI17_OK) return w->st_host->flag;
  return w->st_host->active ? BRI17_ERR_NOT_CONVERGED : BRI17_OK;
}

static int read_state(CgWork* w) {
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->st_host, w->st, sizeof(CgState),
                                 cudaMemcpyDeviceToHost, w->stream));
  BRI17_CUDA_TRY(cudaStreamSynchronize(w->stream));
  return BRI17_OK;
}

// x <- x - mean(x) per component (FP64).
static void project_mean(bri17_op* op, CgWork* w, double* a) {
  const int64_t size = op->g.size;
  int gb = red_blocks(size);
  if (gb > kRedMaxBlocks / 1) gb = kRedMaxBlocks;
  dim3 grid(gb, op->g.dim);
  k_comp_mean<<<grid, kRedThreads, 0, w->stream>>>(a, size, w->st, w->partials);
  dim3 grid2(grid1(size), op->g.dim);
  k_sub_mean<<<grid2, 256, 0, w->stream>>>(a, size, w->st);
}

// r = b - K x (FP64 accurate; the mixed solvers' in float pairs where
// prepare_accurate_residual enabled them).
static int residual64(bri17_op* op, CgWork* w, const double* b, bool mixed = false) {
  int rc = mixed ? apply_accurate_async(op, w->x, w->q, w->stream)
                 : apply_stiffness_async(op, w->x, w->q, w->stream);
  if (rc != BRI17_OK) return rc;
  k_residual<<<grid1(w->n), 256, 0, w->stream>>>(w->r, b, w->q, w->n);
  return BRI17_OK;
}

static int solve_plain64(bri17_op* op, const double* b, double* x, double tol,
                         int maxit, bri17_cg_info* info) {
  CgWork* w;
  int rc = ensure_work(op, false, &w);
  if (rc != BRI17_OK) return rc;
  const int64_t n = w->n;
  cudaStream_t s = w->stream;
  const int rb = red_blocks(n);
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->x, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  const double bb = w->st_host->aux;
  if (!isfinite(bb)) {
    set_error("right-hand side is not finite");
    info->status = BRI17_ERR_BREAKDOWN;
    return BRI17_ERR_BREAKDOWN;
  }
  if (!(bb > 0.0)) {
    // b = 0: the mean-free solution is x = 0.
    BRI17_CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    BRI17_CUDA_TRY(cudaStreamSynchronize(s));
    info->iterations = 0;
    info->outer_iterations = 1;
    info->rel_residual = 0.0;
    info->status = BRI17_OK;
    return BRI17_OK;
  }
  rc = residual64(op, w, b);
  if (rc != BRI17_OK) return rc;
  // aux must hold b.b for k_start's threshold.
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  k_start<double><<<rb, kRedThreads, 0, s>>>(w->r, w->p, n, w->st, w->partials, tol * tol);
  // The recursive residual can stop tracking the true one once the true one
  // reaches what FP64 resolves: below that the recursion may stall above a
  // tolerance that cannot be met, or run on while the iterate drifts and
  // even diverges.  So the true residual |b - K x| is computed (K x into q,
  // which each iteration overwrites anyway) whenever the recursive one has
  // dropped 100x since the last check, and at least every kCheck
  // iterations; the iterate with the smallest true residual is kept.  The
  // solve succeeds when the true residual meets tol.  When the recursive
  // residual has met tol but the true one has not, the true residual
  // replaces it and the CG goes on; the solve stops as stagnated, returning
  // the kept iterate, when that happens again without the true residual
  // having halved since the replacement, when the true residual has not
  // halved over kStallChecks checks while the recursive one sits 10x or
  // more below it (or it has grown past 4x the last halving), over
  // 2 kStallChecks checks in any case, or when it has grown past 10x its
  // smallest.
  constexpr int kCheck = 256;
  constexpr int kStallChecks = 4;
  int iters = 0;
  int status = BRI17_ERR_NOT_CONVERGED;
  double best = INFINITY, prog = INFINITY;
  double replaced = INFINITY;  // squared true residual at the last replacement
  int since_prog = 0;
  bool have_best = false;
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  const double thresh_tol = tol * tol * bb;
  const bool start_active = w->st_host->active != 0;
  if (!start_active)  // converged at the start, or a breakdown
    status = w->st_host->flag != BRI17_OK ? w->st_host->flag : BRI17_OK;
  for (int budget = 0; start_active;) {
    k_plain_resume<<<1, 1, 0, s>>>(w->st, std::max(thresh_tol, 1e-4 * w->st_host->rr));
    budget = (int)std::min<int64_t>(maxit, (int64_t)iters + kCheck);
    // BRI17_OK here: paused at the threshold (a 100x drop, or tol).
    status = run_cg<double>(op, w, w->x, w->r, w->p, w->q, &w->graph64, &w->epoch64, budget,
                            &iters);
    if ((status != BRI17_OK && status != BRI17_ERR_NOT_CONVERGED) ||
        (status == BRI17_ERR_NOT_CONVERGED && iters >= maxit))
      break;
    rc = apply_stiffness_async(op, w->x, w->q, s);
    if (rc != BRI17_OK) return rc;
    k_resnorm<<<rb, kRedThreads, 0, s>>>(b, w->q, n, w->st, w->partials);
    rc = read_state(w);
    if (rc != BRI17_OK) return rc;
    const double rt = w->st_host->aux, rr = w->st_host->rr;
    if (!isfinite(rt)) {
      status = BRI17_ERR_BREAKDOWN;
      break;
    }
    if (rt <= thresh_tol) {
      status = BRI17_OK;
      have_best = false;  // the current iterate is the answer
      break;
    }
    if (rt < best) {
      best = rt;
      have_best = true;
      BRI17_CUDA_TRY(cudaMemcpyAsync(w->xbest, w->x, n * sizeof(double),
                                     cudaMemcpyDeviceToDevice, s));
    }
    if (rr <= thresh_tol) {  // the recursion met tol, the true residual did not
      if (rt >= 0.25 * replaced) {  // and a replacement did not halve it
        status = BRI17_ERR_STAGNATED;
        break;
      }
      // Residual replacement (van der Vorst and Ye, 2000): r = b - K x from
      // the K x just computed, rr = |r|^2, search direction kept; the CG
      // runs on towards tol from the true residual.
      replaced = rt;
      k_residual<<<grid1(n), 256, 0, s>>>(w->r, b, w->q, n);
      k_reliable_resume<<<1, 1, 0, s>>>(w->st, thresh_tol);
      w->st_host->rr = rt;
      continue;
    }
    if (rt < 0.25 * prog) {
      prog = rt;
      since_prog = 0;
    } else if (++since_prog >= kStallChecks &&
               (rr < 0.01 * rt || rt > 16.0 * prog || since_prog >= 2 * kStallChecks)) {
      status = BRI17_ERR_STAGNATED;
      break;
    }
    if (rt > 100.0 * best) {
      status = BRI17_ERR_STAGNATED;
      break;
    }
    if (iters >= maxit) {
      status = BRI17_ERR_NOT_CONVERGED;
      break;
    }
  }
  if (status == BRI17_ERR_STAGNATED && have_best)
    BRI17_CUDA_TRY(cudaMemcpyAsync(w->x, w->xbest, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                   s));
  if (status == BRI17_ERR_CUDA || status == BRI17_ERR_OUT_OF_MEMORY) return status;
  if (status == BRI17_ERR_STAGNATED)
    set_error("the true CG residual stopped decreasing above tol (FP64 cannot resolve tol)");
  project_mean(op, w, w->x);
  rc = residual64(op, w, b);
  if (rc != BRI17_OK) return rc;
  k_dot<double><<<rb, kRedThreads, 0, s>>>(w->r, w->r, n, w->st, w->partials);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  info->iterations = iters;
  info->outer_iterations = 1;
  info->rel_residual = sqrt(w->st_host->aux / bb);
  if (status == BRI17_OK && !(info->rel_residual <= tol * 1.0000001 + 1e-300)) {
    // The recursive residual met tol but the recomputed one did not: the
    // true residual has stagnated at the accuracy rounding allows.
    set_error("the recursive CG residual met tol but the recomputed FP64 residual did not");
    status = BRI17_ERR_STAGNATED;
  }
  info->status = status;
  BRI17_CUDA_TRY(cudaMemcpyAsync(x, w->x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  BRI17_CUDA_TRY(cudaStreamSynchronize(s));
  return status;
}

__global__ void k_residual_f32(float* __restrict__ r, const double* __restrict__ b,
                               const float* __restrict__ kx, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = (float)(b[i] - (double)kx[i]);
}

__global__ void k_f64_to_f32(float* out, const double* in, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// Plain CG on an FP32 handle: FP32 vectors and operator; b and x are FP64
// at the interface.
static int solve_plain32(bri17_op* op, const double* b, double* x, double tol,
                         int maxit, bri17_cg_info* info) {
  CgWork* w;
  int rc = ensure_work(op, false, &w);
  if (rc != BRI17_OK) return rc;
  const int64_t n = w->n;
  cudaStream_t s = w->stream;
  const int rb = red_blocks(n);
  k_f64_to_f32<<<grid1(n), 256, 0, s>>>(w->d32, x, n);
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  const double bb = w->st_host->aux;
  if (!isfinite(bb)) {
    set_error("right-hand side is not finite");
    return BRI17_ERR_BREAKDOWN;
  }
  rc = apply_stiffness_async(op, w->d32, w->q32, s);
  if (rc != BRI17_OK) return rc;
  // r32 = b - K x32 (the product taken in FP32).
  k_residual_f32<<<grid1(n), 256, 0, s>>>(w->r32, b, w->q32, n);
  // aux = b.b for the stopping threshold.
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  k_start<float><<<rb, kRedThreads, 0, s>>>(w->r32, w->p32, n, w->st, w->partials, tol * tol);
  int iters = 0;
  int status = run_cg<float>(op, w, w->d32, w->r32, w->p32, w->q32, &w->graph32,
                             &w->epoch32, maxit, &iters);
  if (status == BRI17_ERR_CUDA || status == BRI17_ERR_OUT_OF_MEMORY) return status;
  BRI17_CUDA_TRY(cudaMemsetAsync(w->x, 0, n * sizeof(double), s));
  k_add_f32<<<grid1(n), 256, 0, s>>>(w->x, w->d32, 1.0, n);
  project_mean(op, w, w->x);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  info->iterations = iters;
  info->outer_iterations = 1;
  info->rel_residual = bb > 0 ? sqrt(w->st_host->rr / bb) : 0.0;
  info->status = status;
  BRI17_CUDA_TRY(cudaMemcpyAsync(x, w->x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  BRI17_CUDA_TRY(cudaStreamSynchronize(s));
  return status;
}

// Mixed precision: FP64 outer refinement around an FP32 CG.
static int solve_mixed(bri17_op* op, const double* b, double* x, double tol,
                       int maxit, bri17_cg_info* info) {
  if (op->precision != BRI17_F64) {
    set_error("mixed-precision CG needs an FP64 handle");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  if (!op->twin32) {
    int shape[3] = {op->g.n[0], op->g.n[1], op->g.n[2]};
    int rc = bri17_op_create(op->g.dim, shape, op->L, op->mu, op->nu, BRI17_F32,
                             &op->twin32);
    if (rc != BRI17_OK) return rc;
  }
  bri17_op* op32 = op->twin32;
  CgWork* w;
  int rc = ensure_work(op, true, &w);
  if (rc != BRI17_OK) return rc;
  rc = prepare_accurate_residual(op);
  if (rc != BRI17_OK) return rc;
  const int64_t n = w->n;
  cudaStream_t s = w->stream;
  const int rb = red_blocks(n);
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->x, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  const double bb = w->st_host->aux;
  info->iterations = 0;
  info->outer_iterations = 0;
  if (!isfinite(bb)) {
    set_error("right-hand side is not finite");
    return BRI17_ERR_BREAKDOWN;
  }
  if (!(bb > 0.0)) {
    BRI17_CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    BRI17_CUDA_TRY(cudaStreamSynchronize(s));
    info->rel_residual = 0.0;
    info->status = BRI17_OK;
    return BRI17_OK;
  }
  int status = BRI17_ERR_NOT_CONVERGED;
  int total = 0;
  double rel = 1.0;
  const int max_outer = 40;
  for (int outer = 0; outer <= max_outer; outer++) {
    project_mean(op, w, w->x);
    rc = residual64(op, w, b, true);
    if (rc != BRI17_OK) return rc;
    project_mean(op, w, w->r);
    k_dot<double><<<rb, kRedThreads, 0, s>>>(w->r, w->r, n, w->st, w->partials);
    rc = read_state(w);
    if (rc != BRI17_OK) return rc;
    const double rr = w->st_host->aux;
    if (!isfinite(rr)) {
      status = BRI17_ERR_BREAKDOWN;
      break;
    }
    rel = sqrt(rr / bb);
    if (rel <= tol) {
      status = BRI17_OK;
      break;
    }
    if (total >= maxit || outer == max_outer) {
      status = BRI17_ERR_NOT_CONVERGED;
      break;
    }
    info->outer_iterations = outer + 1;
    // Inner: K d = r / ||r|| in FP32, to a relative residual that gains
    // what is still needed (at most 1e-5, what FP32 resolves reliably).
    double tin = 0.1 * tol / rel;
    if (tin < 1e-5) tin = 1e-5;
    if (tin > 1e-2) tin = 1e-2;
    const double nr = sqrt(rr);
    k_to_f32<<<grid1(n), 256, 0, s>>>(w->r32, w->r, 1.0 / nr, n);
    BRI17_CUDA_TRY(cudaMemsetAsync(w->d32, 0, n * sizeof(float), s));
    k_dot<float><<<rb, kRedThreads, 0, s>>>(w->r32, w->r32, n, w->st, w->partials);
    k_start<float><<<rb, kRedThreads, 0, s>>>(w->r32, w->p32, n, w->st, w->partials,
                                             tin * tin);
    int iters = 0;
    int st = run_cg<float>(op32, w, w->d32, w->r32, w->p32, w->q32, &w->graph32,
                           &w->epoch32, maxit - total, &iters);
    total += iters;
    if (st == BRI17_ERR_CUDA || st == BRI17_ERR_OUT_OF_MEMORY) return st;
    if (st == BRI17_ERR_TIMEOUT) {  // the FP32 correction is invalid: not folded in
      status = st;
      break;
    }
    if (st == BRI17_ERR_BREAKDOWN && iters == 0) {
      status = BRI17_ERR_BREAKDOWN;
      break;
    }
    k_add_f32<<<grid1(n), 256, 0, s>>>(w->x, w->d32, nr, n);
  }
  info->iterations = total;
  info->rel_residual = rel;
  info->status = status;
  BRI17_CUDA_TRY(cudaMemcpyAsync(x, w->x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  BRI17_CUDA_TRY(cudaStreamSynchronize(s));
  return status;
}

// Mixed precision with reliable updates (Clark et al., "Solving lattice
// QCD systems of equations using mixed precision solvers on GPUs", 2010):
// one FP32 CG whose search direction is kept throughout; whenever its
// recursive residual has dropped by kDelta since the last update (or meets
// the tolerance), the FP32 correction is folded into the FP64 iterate, the
// residual is recomputed in FP64 (r = b - K x, zero-mean projection) and
// replaces the FP32 one.  The solve stops on the FP64 residual.
static int solve_mixed_reliable(bri17_op* op, const double* b, double* x, double tol,
                                int maxit, bri17_cg_info* info) {
  constexpr double kDelta = 0.1;
  constexpr int kStallUpdates = 4;
  if (op->precision != BRI17_F64) {
    set_error("mixed-precision CG needs an FP64 handle");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  if (!op->twin32) {
    int shape[3] = {op->g.n[0], op->g.n[1], op->g.n[2]};
    int rc = bri17_op_create(op->g.dim, shape, op->L, op->mu, op->nu, BRI17_F32,
                             &op->twin32);
    if (rc != BRI17_OK) return rc;
  }
  bri17_op* op32 = op->twin32;
  CgWork* w;
  int rc = ensure_work(op, true, &w);
  if (rc != BRI17_OK) return rc;
  rc = prepare_accurate_residual(op);
  if (rc != BRI17_OK) return rc;
  const int64_t n = w->n;
  cudaStream_t s = w->stream;
  const int rb = red_blocks(n);
  BRI17_CUDA_TRY(cudaMemcpyAsync(w->x, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
  rc = read_state(w);
  if (rc != BRI17_OK) return rc;
  const double bb = w->st_host->aux;
  info->iterations = 0;
  info->outer_iterations = 0;
  if (!isfinite(bb)) {
    set_error("right-hand side is not finite");
    return BRI17_ERR_BREAKDOWN;
  }
  if (!(bb > 0.0)) {
    BRI17_CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    BRI17_CUDA_TRY(cudaStreamSynchronize(s));
    info->rel_residual = 0.0;
    info->status = BRI17_OK;
    return BRI17_OK;
  }
  // r = b - K x (FP64), projected; FP32 copies; p = r32; d = 0.
  auto true_residual = [&](double* rr_out) -> int {
    project_mean(op, w, w->x);
    int e = residual64(op, w, b, true);
    if (e != BRI17_OK) return e;
    project_mean(op, w, w->r);
    k_dot<double><<<rb, kRedThreads, 0, s>>>(w->r, w->r, n, w->st, w->partials);
    e = read_state(w);
    if (e != BRI17_OK) return e;
    *rr_out = w->st_host->aux;
    return BRI17_OK;
  };
  double rr64;
  rc = true_residual(&rr64);
  if (rc != BRI17_OK) return rc;
  double rel = sqrt(rr64 / bb);
  int status = BRI17_ERR_NOT_CONVERGED;
  if (rel <= tol) status = BRI17_OK;
  if (status != BRI17_OK) {
    // The FP32 vectors carry the residual scaled to unit norm (r32 = r / sig,
    // d32 and p32 in the same units), so that their products stay far from
    // FP32 underflow however small the FP64 residual gets.
    double sig = sqrt(rr64);
    k_to_f32<<<grid1(n), 256, 0, s>>>(w->r32, w->r, 1.0 / sig, n);
    BRI17_CUDA_TRY(cudaMemsetAsync(w->d32, 0, n * sizeof(float), s));
    // aux = b.b, so that k_start's threshold is tol^2 b.b / sig^2 (the
    // stopping test in the scaled units).
    k_dot<double><<<rb, kRedThreads, 0, s>>>(b, b, n, w->st, w->partials);
    k_start<float><<<rb, kRedThreads, 0, s>>>(w->r32, w->p32, n, w->st, w->partials,
                                             tol * tol / rr64);
    rc = get_graph<float>(op32, w, w->d32, w->r32, w->p32, w->q32, &w->graph32, &w->epoch32);
    if (rc != BRI17_OK) return rc;
    rc = read_state(w);
    if (rc != BRI17_OK) return rc;
    double rmax2 = rr64;  // squared norm at the last reliable update
    double best2 = rr64;  // smallest squared FP64 residual so far
    int stalled = 0;      // consecutive reliable updates that did not halve it
    int total = 0;
    int breakdowns = 0;  // consecutive FP32 breakdowns (p.Kp <= 0 or NaN)
    while (true) {
      BRI17_CUDA_TRY(cudaGraphLaunch(w->graph32, s));
      BRI17_CUDA_TRY(cudaStreamSynchronize(s));
      const CgState h = *w->st_host;
      total = h.iters;
      if (take_status(op) != BRI17_OK) {
        // A bounded device wait of the chunk ran out: its FP32 work is
        // invalid; the FP64 iterate is kept as it was at the last update.
        status = BRI17_ERR_TIMEOUT;
        break;
      }
      if (h.flag != BRI17_OK) {
        // An FP32 breakdown is answered by a reliable update; two in a row
        // without progress end the solve.
        if (++breakdowns > 2) {
          status = BRI17_ERR_BREAKDOWN;
          break;
        }
      } else {
        breakdowns = 0;
      }
      const bool dropped = h.rr * sig * sig < kDelta * kDelta * rmax2;
      const bool budget = total >= maxit;
      if (!(dropped || !h.active || budget)) continue;
      // Reliable update: x += sig d (FP64), r = b - K x (FP64), r32 = r / sig'.
      k_add_f32<<<grid1(n), 256, 0, s>>>(w->x, w->d32, sig, n);
      BRI17_CUDA_TRY(cudaMemsetAsync(w->d32, 0, n * sizeof(float), s));
      rc = true_residual(&rr64);
      if (rc != BRI17_OK) return rc;
      info->outer_iterations += 1;
      if (!isfinite(rr64)) {
        status = BRI17_ERR_BREAKDOWN;
        break;
      }
      rel = sqrt(rr64 / bb);
      if (rel <= tol) {
        status = BRI17_OK;
        break;
      }
      if (budget) {
        status = BRI17_ERR_NOT_CONVERGED;
        break;
      }
      // Stagnation: each update follows a 10x drop of the FP32 residual, so
      // the FP64 one falls by about as much while it can; kStallUpdates
      // updates in a row that do not halve the best FP64 residual mean that
      // tol lies below what the FP64 residual computation resolves.
      if (rr64 < 0.25 * best2) {
        best2 = rr64;
        stalled = 0;
      } else if (++stalled >= kStallUpdates) {
        set_error("the FP64 residual stopped decreasing above tol");
        status = BRI17_ERR_STAGNATED;
        break;
      }
      // The search direction is kept (rescaled to the new units) while the
      // recomputed residual is close to the recursive one.  Once they part
      // (the FP32 recursion has run below what the FP64 residual resolves:
      // the recomputed residual is rounding noise), p no longer fits r and
      // alpha = r.r / p.Kp would be wrong: CG restarts from p = r when the
      // gap between the two exceeds half the recomputed residual.
      rmax2 = rr64;
      const double sig_new = sqrt(rr64);
      k_gap<<<rb, kRedThreads, 0, s>>>(w->r, w->r32, 1.0 / sig_new, sig / sig_new, n, w->st,
                                       w->partials);
      rc = read_state(w);
      if (rc != BRI17_OK) return rc;
      const bool restart = !(w->st_host->aux <= 0.25);
      k_to_f32<<<grid1(n), 256, 0, s>>>(w->r32, w->r, 1.0 / sig_new, n);
      if (restart)
        BRI17_CUDA_TRY(cudaMemcpyAsync(w->p32, w->r32, n * sizeof(float),
                                       cudaMemcpyDeviceToDevice, s));
      else
        k_scale_f32<<<grid1(n), 256, 0, s>>>(w->p32, (float)(sig / sig_new), n);
      sig = sig_new;
      k_dot<float><<<rb, kRedThreads, 0, s>>>(w->r32, w->r32, n, w->st, w->partials);
      k_reliable_resume<<<1, 1, 0, s>>>(w->st, tol * tol * bb / rr64);
      rc = read_state(w);
      if (rc != BRI17_OK) return rc;
      if (!w->st_host->active) {
        status = BRI17_ERR_BREAKDOWN;
        break;
      }
    }
    info->iterations = total;
  }
  info->rel_residual = rel;
  info->status = status;
  BRI17_CUDA_TRY(cudaMemcpyAsync(x, w->x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  BRI17_CUDA_TRY(cudaStreamSynchronize(s));
  return status;
}

}  // namespace bri17gb

using namespace bri17gb;

extern "C" int bri17_cg_solve(bri17_op* op, const double* b, double* x,
                              double tol, int max_iterations, int mode,
                              bri17_cg_info* info, void* stream) {
  bri17_cg_info dummy;
  if (!info) info = &dummy;
  memset(info, 0, sizeof(*info));
  if (!op || !b || !x) {
    set_error("null pointer");
    return info->status = BRI17_ERR_INVALID_ARGUMENT;
  }
  if (!(tol > 0) || max_iterations < 0 ||
      (mode != BRI17_CG_PLAIN && mode != BRI17_CG_MIXED && mode != BRI17_CG_MIXED_RESTART)) {
    set_error("tol must be > 0, max_iterations >= 0, mode PLAIN, MIXED or MIXED_RESTART");
    return info->status = BRI17_ERR_INVALID_ARGUMENT;
  }
  const int dc = check_device(op);
  if (dc != BRI17_OK) return info->status = dc;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return info->status = cuda_fail(e, "cudaStreamSynchronize");
  const int ts = take_status(op);  // a failure of earlier work on the handle
  if (ts != BRI17_OK) return info->status = ts;
  int rc;
  if (mode == BRI17_CG_MIXED)
    rc = solve_mixed_reliable(op, b, x, tol, max_iterations, info);
  else if (mode == BRI17_CG_MIXED_RESTART)
    rc = solve_mixed(op, b, x, tol, max_iterations, info);
  else if (op->precision == BRI17_F64)
    rc = solve_plain64(op, b, x, tol, max_iterations, info);
  else
    rc = solve_plain32(op, b, x, tol, max_iterations, info);
  info->status = rc;
  return rc;
}
