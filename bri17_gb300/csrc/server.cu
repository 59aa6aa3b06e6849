// server.cu -- continuous-batching server of periodic eigenstress solves.
//
// New (no reference counterpart; the reference solves one mode at a time,
// include/bri17/bri17.hpp:308-355 driven by the Python loop of
// python/demo.py:34-40).
//
// Requests are grouped by geometry (shape, L) into buckets.  A bucket owns
// S slots of device vectors and runs ONE batched mixed-precision CG over all
// its slots: every iteration is one batched FP32 operator application (the
// five FFT passes cover all slots; per-slot materials come from a device
// table) plus batched vector kernels with per-slot scalars, and a chunk of
// iterations is replayed as a CUDA graph.  Converged or empty slots are
// masked on the device (their CTAs exit at once), so requests that arrive
// while others run are admitted into free slots without re-capturing.
// Each bucket has its own stream and progresses on its own: a step retires
// whichever chunks have completed and relaunches those buckets at once, so
// buckets of different sizes overlap on the GPU and small ones are not held
// to the pace of large ones.
//
// Per request (as bri17_cg_solve's mixed mode): b = RHS(tau), x = 0, one FP32
// CG whose search direction is kept throughout; each time its recursive
// residual has dropped 10x the slot pauses for an FP64 reliable update:
// x += d, r = b - K x (FP64), zero-mean projection, stop if ||r|| <= tol
// ||b||, else the FP32 residual is replaced by r and the slot resumes.
// Admission is by device footprint: a new bucket is created only while the
// server's total allocation stays within its memory budget.
#include <math.h>

#include <cmath>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <thread>
#include <deque>
#include <unordered_map>
#include <vector>

#include "op.cuh"
#include "reduce.cuh"

namespace bri17gb {
namespace {

constexpr int kSrvChunk = 16;  // inner iterations per graph replay
// Reliable update when |r32|^2 < kDelta2 |r64|^2, i.e. after a 100x drop of
// the FP32 residual.  On the cubic serving grids (cells of equal sides) the
// FP32 CG drifts little: against a 10x drop the 512-request stream ran at
// 50.0 instead of 46.6 solves/s with the same results.  The single-solve CG
// keeps 10x: on the 512x512x128 grid with cells of aspect 2 a 100x drop
// cost 10% more iterations (3493 against 3165).
constexpr double kDelta2 = 1e-4;

struct Request {
  int64_t id;
  int shape[3];
  double L[3];
  double mu, nu;
  std::vector<double> tau;  // 6 x size (copied at submit)
  const double* tau_borrowed = nullptr;  // or the caller's buffer (borrowed submit)
  double* x_host;
  bool x_locked = false;   // x_host is page-locked: the result copy is asynchronous
  cudaEvent_t done_ev = nullptr;  // that copy's completion
  int final_status = BRI17_OK;
  double tol;
  int max_iterations;
  double t_submit = 0, t_admit = 0, t_finish = 0;
  int iters = 0, outer = 0, breakdowns = 0;
  double bb = 0, rel = 1, nr = 0;
  double mat64[2] = {0, 0};  // upload sources (live until the copies ran)
  float mat32[2] = {0, 0};
  float matdf[4] = {0, 0, 0, 0};  // (s, mu) as float pairs (hi, lo)
  int status = BRI17_OK;
  bool cancel = false;
};

// kInner: the slot's FP32 CG runs in the bucket's chunks.  kOuter: its FP64
// outer residual has been enqueued; the decision (retire or restart) is
// taken when the stream work that computes it has completed.
enum SlotState { kFree = 0, kInner = 1, kOuter = 2 };

struct Bucket {
  int shape[3];
  double L[3];
  int S = 0;
  int64_t size = 0, n = 0;
  bri17_op* op32 = nullptr;
  bri17_op* op64 = nullptr;
  double *b = nullptr, *x = nullptr, *r = nullptr, *q64 = nullptr, *tau = nullptr;
  float *d = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr;
  float* mat32 = nullptr;
  double* mat64 = nullptr;
  float* matdf = nullptr;  // per slot (s, mu) as float pairs, for float-pair residuals
  void* spec32 = nullptr;
  CgState* st = nullptr;
  CgState* st_host = nullptr;
  double* partials = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<int> slot_state;
  std::vector<Request*> slot_req;
  int64_t bytes = 0;
  bool in_flight = false;  // work was enqueued on the stream and not yet retired
  bool enqueued = false;   // work enqueued since the last launch decision
};

// --- batched CG kernels: grid (blocks, S), slot z = blockIdx.y -----------

__device__ __forceinline__ double slot_block_total(double v, double* partials,
                                                   unsigned int* counter,
                                                   int nparts, double* total,
                                                   bool* last) {
  __shared__ bool is_last;
  const double b = block_sum(v);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == (unsigned int)nparts - 1);
  }
  __syncthreads();
  *last = is_last;
  if (!is_last) return 0.0;
  __threadfence();
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += __ldcg(partials + i);
  const double tot = block_sum(s);
  if (threadIdx.x == 0) {
    *total = tot;
    *counter = 0u;
  }
  return tot;
}

__global__ void __launch_bounds__(kRedThreads)
    kb_dot_pq(const float* __restrict__ p, const float* __restrict__ q, int64_t n,
              CgState* sts, double* partials) {
  CgState* st = sts + blockIdx.y;
  if (!st->active) return;
  const double v = vdot<float>(p + blockIdx.y * n, q + blockIdx.y * n, n,
                               (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                               (int64_t)gridDim.x * blockDim.x);
  double tot;
  bool last;
  slot_block_total(v, partials + blockIdx.y * kRedMaxBlocks, &st->counter, gridDim.x,
                   &tot, &last);
  if (last && threadIdx.x == 0) {
    st->pq = tot;
    if (!(tot > 0.0) || !isfinite(tot)) {
      st->flag = BRI17_ERR_BREAKDOWN;
      st->active = 0;
    } else {
      st->alpha = st->rr / tot;
    }
  }
}

__global__ void __launch_bounds__(kRedThreads)
    kb_update(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
              const float* __restrict__ q, int64_t n, CgState* sts, double* partials,
              int max_iters) {
  CgState* st = sts + blockIdx.y;
  if (!st->active) return;
  const int64_t o = blockIdx.y * n;
  const double v = vupdate<float>(x + o, r + o, p + o, q + o, (float)st->alpha, n,
                                  (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                                  (int64_t)gridDim.x * blockDim.x);
  double tot;
  bool last;
  slot_block_total(v, partials + blockIdx.y * kRedMaxBlocks, &st->counter, gridDim.x,
                   &tot, &last);
  if (last && threadIdx.x == 0) {
    st->iters += 1;
    if (!isfinite(tot)) {
      st->flag = BRI17_ERR_BREAKDOWN;
      st->active = 0;
      return;
    }
    st->beta = tot / st->rr;
    st->rr = tot;
    // Pause for an FP64 reliable update once the FP32 residual has dropped
    // by kDelta since the last one (or meets the tolerance).
    if (tot <= st->thresh || st->iters >= max_iters || tot < kDelta2 * st->rmax2)
      st->pause = 1;
  }
}

__global__ void __launch_bounds__(kRedThreads)
    kb_pupdate(float* __restrict__ p, const float* __restrict__ r, int64_t n,
               const CgState* sts) {
  const CgState* st = sts + blockIdx.y;
  if (!st->active) return;
  const int64_t o = blockIdx.y * n;
  vpupdate<float>(p + o, r + o, (float)st->beta, n,
                  (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                  (int64_t)gridDim.x * blockDim.x);
}

// --- per-slot helpers (one slot, 1-D grids) --------------------------------

__global__ void __launch_bounds__(kRedThreads)
    ks_dot(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
           CgState* st, double* partials) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v += a[i] * b[i];
  double tot;
  bool last;
  slot_block_total(v, partials, &st->counter, gridDim.x, &tot, &last);
  if (last && threadIdx.x == 0) st->aux = tot;
}

// r = b - kx, then subtract per-component means computed in a second kernel.
__global__ void ks_residual(double* __restrict__ r, const double* __restrict__ b,
                            const double* __restrict__ kx, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - kx[i];
}

__global__ void __launch_bounds__(kRedThreads)
    ks_comp_mean(const double* __restrict__ a, int64_t size, CgState* st,
                 double* partials) {
  const double* ac = a + (int64_t)blockIdx.y * size;
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size;
       i += (int64_t)gridDim.x * blockDim.x)
    v += ac[i];
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

__global__ void ks_sub_mean(double* __restrict__ a, int64_t size, const CgState* st) {
  const double m = st->mean[blockIdx.y];
  double* ac = a + (int64_t)blockIdx.y * size;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < size;
       i += (int64_t)gridDim.x * blockDim.x)
    ac[i] -= m;
}

// FP32 CG start: r32 = r, p = r32, d = 0, rr, thresh (tol^2 b.b), rmax2.
__global__ void __launch_bounds__(kRedThreads)
    ks_start(const double* __restrict__ r, float* __restrict__ r32, float* __restrict__ d,
             float* __restrict__ p, int64_t n, CgState* st, double* partials, double thresh,
             double rmax2) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = (float)r[i];
    r32[i] = ri;
    p[i] = ri;
    d[i] = 0.f;
    v += (double)ri * (double)ri;
  }
  double tot;
  bool last;
  slot_block_total(v, partials, &st->counter, gridDim.x, &tot, &last);
  if (last && threadIdx.x == 0) {
    st->rr = tot;
    st->thresh = thresh;
    st->rmax2 = rmax2;
    st->iters = 0;
    st->pause = 0;
    st->flag = isfinite(tot) ? BRI17_OK : BRI17_ERR_BREAKDOWN;
    st->active = (tot > thresh && isfinite(tot)) ? 1 : 0;
  }
}

// Reliable update: the FP32 residual is replaced by the FP64 one, the
// correction restarts from zero, the search direction p is kept.
__global__ void __launch_bounds__(kRedThreads)
    ks_reliable(const double* __restrict__ r, float* __restrict__ r32, float* __restrict__ d,
                int64_t n, CgState* st, double* partials, double rmax2) {
  double v = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = (float)r[i];
    r32[i] = ri;
    d[i] = 0.f;
    v += (double)ri * (double)ri;
  }
  double tot;
  bool last;
  slot_block_total(v, partials, &st->counter, gridDim.x, &tot, &last);
  if (last && threadIdx.x == 0) {
    st->rr = tot;
    st->rmax2 = rmax2;
    st->pause = 0;
    st->flag = isfinite(tot) ? BRI17_OK : BRI17_ERR_BREAKDOWN;
    // At least one more chunk runs, so every update changes the iterate.
    st->active = isfinite(tot) ? 1 : 0;
  }
}

__global__ void ks_axpy32(double* __restrict__ x, const float* __restrict__ d, double a,
                          int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += a * (double)d[i];
}

__global__ void ks_set_inactive(CgState* st) { st->active = 0; }

unsigned g1(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace
}  // namespace bri17gb

using namespace bri17gb;

struct bri17_server {
  int64_t budget = 0;
  int max_active = 8;  // most slots per bucket
  bool size_priority = false;  // smaller geometries' streams first
  int64_t used = 0;
  int64_t next_id = 1;
  std::deque<Request*> queue;
  std::vector<Bucket*> buckets;
  std::vector<bri17_request_result> done;
  std::unordered_map<int64_t, Request*> live;
  std::vector<Request*> finishing;  // solution copies to page-locked x_host in flight
  // Fault injection (bri17_server_inject_alloc_failure): when >= 0, the next
  // bucket creation fails at its work buffer number fail_alloc_at (0-based)
  // as cudaMalloc does when memory runs out.
  int fail_alloc_at = -1;
  std::chrono::steady_clock::time_point t0;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

#define SRV_TRY(expr)                                   \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
  } while (0)

int64_t slot_bytes(int64_t n) { return n * (5 * 8 + 4 * 4); }

constexpr int64_t kBucketDoF = 48ll << 20;

int64_t bucket_bytes(const int* shape, int S) {
  int64_t size = (int64_t)shape[0] * shape[1] * shape[2];
  int64_t n = 3 * size;
  int64_t cspec = (int64_t)shape[0] * shape[1] * (shape[2] / 2 + 1);
  return S * slot_bytes(n) + 6 * size * 8 /* tau staging */ +
         (int64_t)S * 3 * cspec * 8 /* FP32 batched spectrum */ +
         6 * cspec * 16 + 3 * cspec * 8 /* op64 / op32 own spectra */ +
         (int64_t)S * (kRedMaxBlocks * 8 + sizeof(CgState));
}

void free_bucket(Bucket* B) {
  if (!B) return;
  if (B->stream) cudaStreamSynchronize(B->stream);
  if (B->graph) cudaGraphExecDestroy(B->graph);
  bri17_op_destroy(B->op32);
  bri17_op_destroy(B->op64);
  void* ps[] = {B->b, B->x, B->r, B->q64, B->tau, B->d, B->r32, B->p32, B->q32,
                B->mat32, B->mat64, B->matdf, B->spec32, B->st, B->partials};
  for (void* p : ps) cudaFree(p);
  cudaFreeHost(B->st_host);
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
}

int capture_graph(Bucket* B) {
  const int64_t n = B->n;
  const int rb = red_blocks(n);
  cudaStream_t s = B->stream;
  cudaGraph_t g;
  SRV_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = BRI17_OK;
  const int flag_stride = (int)(sizeof(CgState) / sizeof(int));
  const int* flags = &B->st[0].active;
  for (int it = 0; it < kSrvChunk && rc == BRI17_OK; it++) {
    rc = apply_stiffness_batched_async(B->op32, B->S, B->p32, B->q32, B->spec32, B->mat32, s,
                                       flags, flag_stride);
    dim3 grid(rb, B->S);
    kb_dot_pq<<<grid, kRedThreads, 0, s>>>(B->p32, B->q32, n, B->st, B->partials);
    kb_update<<<grid, kRedThreads, 0, s>>>(B->d, B->r32, B->p32, B->q32, n, B->st,
                                           B->partials, 1 << 30);
    dim3 g2(g1(n), B->S);
    kb_pupdate<<<g2, 256, 0, s>>>(B->p32, B->r32, n, B->st);
    k_apply_pause<<<1, 64, 0, s>>>(B->st, B->S);
  }
  cudaMemcpyAsync(B->st_host, B->st, B->S * sizeof(CgState), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc != BRI17_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&B->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return BRI17_OK;
}

int make_bucket(bri17_server* srv, const Request* q, Bucket** out) {
  // Slots: enough for about kBucketDoF unknowns of batched work per
  // iteration (at least 8; small geometries get many slots, so their
  // requests are not queued behind a handful of slots), at most max_active;
  // the axis-1 pass launches S * 3 * n0 CTA rows (grid.y <= 65535).
  const int64_t n_slot = 3 * (int64_t)q->shape[0] * q->shape[1] * q->shape[2];
  const int64_t want = std::max<int64_t>(8, (kBucketDoF + n_slot - 1) / n_slot);
  const int S = (int)std::max<int64_t>(
      1, std::min<int64_t>({(int64_t)srv->max_active, want, 65535 / (3 * q->shape[0])}));
  const int64_t bytes = bucket_bytes(q->shape, S);
  if (srv->used + bytes > srv->budget) return BRI17_ERR_BUSY;
  Bucket* B = new Bucket();
  memcpy(B->shape, q->shape, sizeof(B->shape));
  memcpy(B->L, q->L, sizeof(B->L));
  B->S = S;
  B->size = (int64_t)q->shape[0] * q->shape[1] * q->shape[2];
  B->n = 3 * B->size;
  B->bytes = bytes;
  auto fail = [&](int rc) {
    free_bucket(B);
    return rc;
  };
  int rc = bri17_op_create(3, q->shape, q->L, 1.0, 0.3, BRI17_F32, &B->op32);
  if (rc != BRI17_OK) return fail(rc);
  rc = bri17_op_create(3, q->shape, q->L, 1.0, 0.3, BRI17_F64, &B->op64);
  if (rc != BRI17_OK) return fail(rc);
  rc = ensure_spectrum(B->op64, 6);
  if (rc != BRI17_OK) return fail(rc);
  // Float-pair tables for the slots' FP64 residuals where the grid has
  // float-pair instances; without them (or if building them fails) the
  // residuals stay on the FP64 pipe.
  if (prepare_accurate_residual(B->op64) != BRI17_OK) {
    B->op64->residual_df = false;
    cudaGetLastError();
  }
  const int64_t n = B->n, Sn = S * n;
  const int64_t cspec = B->op32->g.cspec;
  // An injected failure takes the place of work buffer number inject_at.
  const int inject_at = srv->fail_alloc_at;
  srv->fail_alloc_at = -1;
  int alloc_no = 0;
#define ALLOC(p, bytes_)                                                            \
  do {                                                                              \
    cudaError_t _e = alloc_no++ == inject_at ? cudaErrorMemoryAllocation             \
                                             : cudaMalloc((void**)&(p), (bytes_));  \
    if (_e != cudaSuccess) return fail(cuda_fail(_e, "cudaMalloc(bucket)"));        \
  } while (0)
  ALLOC(B->b, Sn * 8);
  ALLOC(B->x, Sn * 8);
  ALLOC(B->r, Sn * 8);
  ALLOC(B->q64, Sn * 8);
  ALLOC(B->tau, 6 * B->size * 8);
  ALLOC(B->d, Sn * 4);
  ALLOC(B->r32, Sn * 4);
  ALLOC(B->p32, Sn * 4);
  ALLOC(B->q32, Sn * 4);
  ALLOC(B->mat32, S * 2 * 4);
  ALLOC(B->mat64, S * 2 * 8);
  ALLOC(B->matdf, S * 4 * 4);
  ALLOC(B->spec32, (int64_t)S * 3 * cspec * 8);
  ALLOC(B->st, S * sizeof(CgState));
  ALLOC(B->partials, (int64_t)S * kRedMaxBlocks * 8);
#undef ALLOC
  if (cudaMallocHost((void**)&B->st_host, S * sizeof(CgState)) != cudaSuccess)
    return fail(cuda_fail(cudaErrorMemoryAllocation, "cudaMallocHost"));
  memset(B->st_host, 0, S * sizeof(CgState));
  if (cudaMemset(B->st, 0, S * sizeof(CgState)) != cudaSuccess ||
      cudaMemset(B->mat32, 0, S * 2 * 4) != cudaSuccess ||
      cudaMemset(B->mat64, 0, S * 2 * 8) != cudaSuccess ||
      cudaMemset(B->matdf, 0, S * 4 * 4) != cudaSuccess ||
      cudaMemset(B->p32, 0, Sn * 4) != cudaSuccess)
    return fail(cuda_fail(cudaErrorUnknown, "cudaMemset(bucket)"));
  // With size priorities on, smaller geometries get higher stream priority:
  // their short kernels are scheduled ahead of the queued CTAs of large
  // buckets' passes (lower latency for small requests, lower throughput).
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  const int levels = least - greatest + 1;
  const double tpos = std::max(0.0, std::log2((double)B->size / 32768.0)) / 6.0;
  const int prio = srv->size_priority
                       ? greatest + std::min(levels - 1, (int)std::lround(tpos * (levels - 1)))
                       : least;
  if (cudaStreamCreateWithPriority(&B->stream, cudaStreamNonBlocking, prio) != cudaSuccess)
    return fail(cuda_fail(cudaErrorUnknown, "cudaStreamCreate"));
  B->slot_state.assign(S, kFree);
  B->slot_req.assign(S, nullptr);
  rc = capture_graph(B);
  if (rc != BRI17_OK) return fail(rc);
  srv->used += bytes;
  srv->buckets.push_back(B);
  *out = B;
  return BRI17_OK;
}

Bucket* find_bucket(bri17_server* srv, const Request* q) {
  for (Bucket* B : srv->buckets)
    if (memcmp(B->shape, q->shape, sizeof(B->shape)) == 0 &&
        memcmp(B->L, q->L, sizeof(B->L)) == 0)
      return B;
  return nullptr;
}

int free_slot(const Bucket* B) {
  for (int z = 0; z < B->S; z++)
    if (B->slot_state[z] == kFree) return z;
  return -1;
}

// Enqueue the FP64 outer residual of slot z: r = b - K x, projected, and
// aux = r.r (read by the caller after a sync).
int enqueue_residual(Bucket* B, int z, bool x_is_zero) {
  const int64_t n = B->n;
  cudaStream_t s = B->stream;
  double* bz = B->b + z * n;
  double* xz = B->x + z * n;
  double* rz = B->r + z * n;
  CgState* st = B->st + z;
  double* parts = B->partials + z * kRedMaxBlocks;
  if (x_is_zero) {
    SRV_TRY(cudaMemcpyAsync(rz, bz, n * 8, cudaMemcpyDeviceToDevice, s));
  } else {
    dim3 gm(std::min(red_blocks(B->size), kRedMaxBlocks / 3), 3);
    ks_comp_mean<<<gm, kRedThreads, 0, s>>>(xz, B->size, st, parts);
    ks_sub_mean<<<dim3(g1(B->size), 3), 256, 0, s>>>(xz, B->size, st);
    // FP64-accurate K x in float pairs where the grid has them (power-of-two
    // strided axes 64..512, last axis 128..1024), else on the FP64 pipe.
    int rc = B->op64->residual_df
                 ? apply_accurate_mat_async(B->op64, xz, B->q64 + z * n, B->matdf + 4 * z, s)
                 : apply_stiffness_batched_async(B->op64, 1, xz, B->q64 + z * n,
                                                 B->op64->spec, B->mat64 + 2 * z, s);
    if (rc != BRI17_OK) return rc;
    ks_residual<<<g1(n), 256, 0, s>>>(rz, bz, B->q64 + z * n, n);
  }
  dim3 gm(std::min(red_blocks(B->size), kRedMaxBlocks / 3), 3);
  ks_comp_mean<<<gm, kRedThreads, 0, s>>>(rz, B->size, st, parts);
  ks_sub_mean<<<dim3(g1(B->size), 3), 256, 0, s>>>(rz, B->size, st);
  ks_dot<<<red_blocks(n), kRedThreads, 0, s>>>(rz, rz, n, st, parts);
  SRV_TRY(cudaMemcpyAsync(&B->st_host[z], st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  return BRI17_OK;
}

void finish(bri17_server* srv, Request* q, int status) {
  q->status = status;
  q->t_finish = srv->now();
  bri17_request_result res;
  res.id = q->id;
  res.status = status;
  res.iterations = q->iters;
  res.outer_iterations = q->outer;
  res.rel_residual = q->rel;
  res.submit_time_s = q->t_submit;
  res.admit_time_s = q->t_admit;
  res.finish_time_s = q->t_finish;
  srv->done.push_back(res);
  srv->live.erase(q->id);
  if (q->done_ev) cudaEventDestroy(q->done_ev);
  delete q;
}

// Admit q into slot z of B: upload tau and material, compute b, x = 0 and
// the initial residual r = b, all enqueued on the bucket's stream; the first
// outer decision (which starts the inner CG) is taken once it has run.
int admit(bri17_server* srv, Bucket* B, int z, Request* q) {
  cudaStream_t s = B->stream;
  const int64_t n = B->n;
  q->t_admit = srv->now();
  // The slot stays masked out of the chunks until its first outer decision.
  ks_set_inactive<<<1, 1, 0, s>>>(B->st + z);
  SRV_TRY(cudaMemcpyAsync(B->tau, q->tau_borrowed ? q->tau_borrowed : q->tau.data(),
                          6 * B->size * 8, cudaMemcpyHostToDevice, s));
  const double corr = B->op64->corr;
  const double scaling = q->mu / (1. - 2. * q->nu);
  q->mat64[0] = scaling * corr;
  q->mat64[1] = q->mu * corr;
  q->mat32[0] = (float)q->mat64[0];
  q->mat32[1] = (float)q->mat64[1];
  SRV_TRY(cudaMemcpyAsync(B->mat64 + 2 * z, q->mat64, sizeof(q->mat64), cudaMemcpyHostToDevice,
                          s));
  SRV_TRY(cudaMemcpyAsync(B->mat32 + 2 * z, q->mat32, sizeof(q->mat32), cudaMemcpyHostToDevice,
                          s));
  if (B->op64->residual_df) {
    const df64 sdf(q->mat64[0]), mdf(q->mat64[1]);
    q->matdf[0] = sdf.hi;
    q->matdf[1] = sdf.lo;
    q->matdf[2] = mdf.hi;
    q->matdf[3] = mdf.lo;
    SRV_TRY(cudaMemcpyAsync(B->matdf + 4 * z, q->matdf, sizeof(q->matdf),
                            cudaMemcpyHostToDevice, s));
  }
  int rc = eigenstress_rhs_batched_async(B->op64, 1, B->tau, B->b + z * n, B->op64->spec, s);
  if (rc != BRI17_OK) return rc;
  SRV_TRY(cudaMemsetAsync(B->x + z * n, 0, n * 8, s));
  // The pageable tau copy has been staged when cudaMemcpyAsync returned; the
  // host copy can go.
  std::vector<double>().swap(q->tau);
  rc = enqueue_residual(B, z, true);
  if (rc != BRI17_OK) return rc;
  B->slot_state[z] = kOuter;
  B->slot_req[z] = q;
  B->enqueued = true;
  return BRI17_OK;
}

// Outer step of slot z after its residual is known (st_host[z].aux = r.r):
// retire or restart the inner CG.  Returns true if the slot stays busy.
int outer_decide(bri17_server* srv, Bucket* B, int z, bool* busy) {
  Request* q = B->slot_req[z];
  const double rr = B->st_host[z].aux;
  if (q->outer == 0) q->bb = rr;  // the initial residual is b
  *busy = false;
  if (!isfinite(rr) || !isfinite(q->bb)) {
    q->rel = NAN;
    B->slot_state[z] = kFree;
    B->slot_req[z] = nullptr;
    finish(srv, q, BRI17_ERR_BREAKDOWN);
    return BRI17_OK;
  }
  q->rel = q->bb > 0 ? sqrt(rr / q->bb) : 0.0;
  const bool converged = q->rel <= q->tol || q->bb == 0.0;
  if (converged || q->iters >= q->max_iterations || q->cancel) {
    const int64_t n = B->n;
    const int status = q->cancel ? BRI17_ERR_CANCELLED
                                 : converged ? BRI17_OK : BRI17_ERR_NOT_CONVERGED;
    SRV_TRY(cudaMemcpyAsync(q->x_host, B->x + z * n, n * 8, cudaMemcpyDeviceToHost,
                            B->stream));
    B->slot_state[z] = kFree;
    B->slot_req[z] = nullptr;
    if (q->x_locked) {
      // The copy runs on the bucket's stream (later work in the slot waits
      // for it); the request finishes when the step sees its event.
      SRV_TRY(cudaEventCreateWithFlags(&q->done_ev, cudaEventDisableTiming));
      SRV_TRY(cudaEventRecord(q->done_ev, B->stream));
      q->final_status = status;
      srv->finishing.push_back(q);
      B->enqueued = true;
      return BRI17_OK;
    }
    SRV_TRY(cudaStreamSynchronize(B->stream));
    finish(srv, q, status);
    return BRI17_OK;
  }
  const int64_t n = B->n;
  if (q->outer == 0) {
    ks_start<<<red_blocks(n), kRedThreads, 0, B->stream>>>(
        B->r + z * n, B->r32 + z * n, B->d + z * n, B->p32 + z * n, n, B->st + z,
        B->partials + z * kRedMaxBlocks, q->tol * q->tol * q->bb, rr);
  } else {
    ks_reliable<<<red_blocks(n), kRedThreads, 0, B->stream>>>(
        B->r + z * n, B->r32 + z * n, B->d + z * n, n, B->st + z,
        B->partials + z * kRedMaxBlocks, rr);
  }
  q->outer += 1;
  B->slot_state[z] = kInner;
  B->enqueued = true;
  *busy = true;
  return BRI17_OK;
}

}  // namespace

extern "C" int bri17_server_create(int64_t budget, int max_active, bri17_server** out) {
  if (!out) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  if (budget <= 0 || max_active < 1 || max_active > 256) {
    set_error("memory budget must be > 0 and max_active in [1, 256]");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return BRI17_ERR_NO_DEVICE;
  }
  bri17_server* s = new bri17_server();
  s->budget = budget;
  s->max_active = max_active;
  s->t0 = std::chrono::steady_clock::now();
  *out = s;
  return BRI17_OK;
}

extern "C" int bri17_server_set_size_priority(bri17_server* srv, int enable) {
  if (!srv) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  srv->size_priority = enable != 0;
  return BRI17_OK;
}

extern "C" int bri17_server_inject_alloc_failure(bri17_server* srv, int at) {
  if (!srv || at < -1) {
    set_error("null server or allocation number below -1");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  srv->fail_alloc_at = at;
  return BRI17_OK;
}

extern "C" int bri17_server_destroy(bri17_server* srv) {
  if (!srv) return BRI17_OK;
  for (Bucket* B : srv->buckets) free_bucket(B);
  for (Request* q : srv->finishing)
    if (q->done_ev) cudaEventDestroy(q->done_ev);
  for (Request* q : srv->queue) delete q;
  for (auto& kv : srv->live)
    if (std::find(srv->queue.begin(), srv->queue.end(), kv.second) == srv->queue.end())
      delete kv.second;
  delete srv;
  return BRI17_OK;
}

namespace {

bool page_locked(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

int submit_request(bri17_server* srv, const int* shape, const double* L, double mu, double nu,
                   const double* tau_host, double* x_host, double tol, int max_iterations,
                   bool borrow, int64_t* id) {
  if (!srv || !shape || !L || !tau_host || !x_host || !id) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < 3; i++)
    if (shape[i] < 1 || shape[i] > 1024 || !(L[i] > 0) || !std::isfinite(L[i])) {
      set_error("shape entries must be in [1, 1024] and L entries positive and finite");
      return BRI17_ERR_INVALID_ARGUMENT;
    }
  if (!(mu > 0) || !std::isfinite(mu) || !(nu > -1.0 && nu < 0.5) || !(tol > 0) ||
      max_iterations < 1) {
    set_error("need finite mu > 0, -1 < nu < 0.5, tol > 0, max_iterations >= 1");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  AxisPlan p;
  for (int i = 0; i < 3; i++)
    if (!make_plan(shape[i], &p)) {
      set_error("axis length has a prime factor above 61");
      return BRI17_ERR_UNSUPPORTED_SIZE;
    }
  if (bucket_bytes(shape, 1) > srv->budget) {
    set_error("request footprint exceeds the server's memory budget");
    return BRI17_ERR_OUT_OF_MEMORY;
  }
  Request* q = new Request();
  q->id = srv->next_id++;
  memcpy(q->shape, shape, sizeof(q->shape));
  memcpy(q->L, L, sizeof(q->L));
  q->mu = mu;
  q->nu = nu;
  const int64_t size = (int64_t)shape[0] * shape[1] * shape[2];
  if (borrow)
    q->tau_borrowed = tau_host;
  else
    q->tau.assign(tau_host, tau_host + 6 * size);
  q->x_host = x_host;
  q->x_locked = page_locked(x_host);
  q->tol = tol;
  q->max_iterations = max_iterations;
  q->t_submit = srv->now();
  srv->queue.push_back(q);
  srv->live[q->id] = q;
  *id = q->id;
  return BRI17_OK;
}

}  // namespace

extern "C" int bri17_server_submit(bri17_server* srv, const int* shape, const double* L,
                                   double mu, double nu, const double* tau_host,
                                   double* x_host, double tol, int max_iterations,
                                   int64_t* id) {
  return submit_request(srv, shape, L, mu, nu, tau_host, x_host, tol, max_iterations, false,
                        id);
}

extern "C" int bri17_server_submit_borrowed(bri17_server* srv, const int* shape,
                                            const double* L, double mu, double nu,
                                            const double* tau_host, double* x_host,
                                            double tol, int max_iterations, int64_t* id) {
  return submit_request(srv, shape, L, mu, nu, tau_host, x_host, tol, max_iterations, true,
                        id);
}

extern "C" int bri17_server_cancel(bri17_server* srv, int64_t id) {
  if (!srv) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  auto it = srv->live.find(id);
  if (it == srv->live.end()) return BRI17_ERR_NOT_FOUND;
  Request* q = it->second;
  for (auto qi = srv->queue.begin(); qi != srv->queue.end(); ++qi)
    if (*qi == q) {
      srv->queue.erase(qi);
      finish(srv, q, BRI17_ERR_CANCELLED);
      return BRI17_OK;
    }
  q->cancel = true;  // running: retired at the next step
  return BRI17_OK;
}

namespace {

// Retire side of one bucket whose enqueued work has completed.
//  (a) Slots whose FP64 outer residual was enqueued: decide (retire the
//      request, or restart its inner CG with a reliable update).
//  (b) Slots whose inner CG stopped in the last chunk: x += d, enqueue the
//      FP64 outer residual (decided at the next retire).
// Nothing here waits for the stream, except the copy of a finished
// request's solution to its host buffer.
int retire(bri17_server* srv, Bucket* B) {
  std::vector<int> outer_before, inner_before;
  for (int z = 0; z < B->S; z++) {
    if (B->slot_state[z] == kOuter) outer_before.push_back(z);
    if (B->slot_state[z] == kInner) inner_before.push_back(z);
  }
  for (int z : outer_before) {
    bool busy;
    const int rc = outer_decide(srv, B, z, &busy);
    if (rc != BRI17_OK) return rc;
  }
  for (int z : inner_before) {
    Request* q = B->slot_req[z];
    const CgState& h = B->st_host[z];
    if (q->cancel && h.active) {
      ks_set_inactive<<<1, 1, 0, B->stream>>>(B->st + z);
      B->enqueued = true;
    }
    if (!h.active || q->cancel) {
      q->iters = h.iters;  // cumulative: reliable updates keep the count
      q->breakdowns = h.flag != BRI17_OK ? q->breakdowns + 1 : 0;
      if (q->breakdowns > 2) {
        q->rel = NAN;
        B->slot_state[z] = kFree;
        B->slot_req[z] = nullptr;
        finish(srv, q, BRI17_ERR_BREAKDOWN);
        continue;
      }
      ks_axpy32<<<g1(B->n), 256, 0, B->stream>>>(B->x + z * B->n, B->d + z * B->n, 1.0, B->n);
      const int rc = enqueue_residual(B, z, false);
      if (rc != BRI17_OK) return rc;
      B->slot_state[z] = kOuter;
      B->enqueued = true;
    } else if (h.iters >= q->max_iterations) {
      ks_set_inactive<<<1, 1, 0, B->stream>>>(B->st + z);
      B->enqueued = true;
    }
  }
  return BRI17_OK;
}

bool bucket_has_inner(const Bucket* B) {
  for (int z = 0; z < B->S; z++)
    if (B->slot_state[z] == kInner) return true;
  return false;
}

}  // namespace

// Buckets progress independently: a bucket's chunk (kSrvChunk CG
// iterations of all its slots, one graph) is relaunched as soon as the
// previous one has completed and been retired, so small geometries are not
// held to the pace of large ones.  A step does not wait for chunks; when it
// finds nothing to do it waits (bounded, about 0.2 ms) for any chunk to
// complete before returning.
extern "C" int bri17_server_step(bri17_server* srv, int* active) {
  if (!srv) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  bool progress = false;
  // 0. Requests whose solution copy to a page-locked buffer has completed.
  for (size_t i = 0; i < srv->finishing.size();) {
    Request* q = srv->finishing[i];
    const cudaError_t qs = cudaEventQuery(q->done_ev);
    if (qs == cudaErrorNotReady) {
      i++;
      continue;
    }
    if (qs != cudaSuccess) return cuda_fail(qs, "server result copy");
    srv->finishing.erase(srv->finishing.begin() + i);
    finish(srv, q, q->final_status);
    progress = true;
  }
  // 1. Retire completed chunks.
  for (Bucket* B : srv->buckets) {
    if (!B->in_flight) continue;
    const cudaError_t qs = cudaStreamQuery(B->stream);
    if (qs == cudaErrorNotReady) continue;
    if (qs != cudaSuccess) return cuda_fail(qs, "server chunk");
    B->in_flight = false;
    progress = true;
    if (take_status(B->op32) != BRI17_OK) {
      // A bounded device wait of the chunk ran out: the chunk's FP32 work is
      // invalid for every slot that was iterating; those requests fail.
      for (int z = 0; z < B->S; z++) {
        if (B->slot_state[z] != kInner) continue;
        ks_set_inactive<<<1, 1, 0, B->stream>>>(B->st + z);
        Request* q = B->slot_req[z];
        q->iters = B->st_host[z].iters;
        q->rel = NAN;
        B->slot_state[z] = kFree;
        B->slot_req[z] = nullptr;
        finish(srv, q, BRI17_ERR_TIMEOUT);
        B->enqueued = true;
      }
    }
    const int rc = retire(srv, B);
    if (rc != BRI17_OK) return rc;
  }
  // 2. Admission: FIFO, skipping requests whose bucket is full or has a
  //    chunk in flight (no head-of-line blocking across geometries).
  for (auto it = srv->queue.begin(); it != srv->queue.end();) {
    Request* q = *it;
    Bucket* B = find_bucket(srv, q);
    if (!B) {
      int rc = make_bucket(srv, q, &B);
      if (rc == BRI17_ERR_BUSY) {
        // Release an idle bucket of another geometry, then retry once.
        for (size_t i = 0; i < srv->buckets.size(); i++) {
          Bucket* E = srv->buckets[i];
          bool idle = !E->in_flight;
          for (int z = 0; z < E->S; z++) idle = idle && E->slot_state[z] == kFree;
          if (idle) {
            srv->used -= E->bytes;
            free_bucket(E);
            srv->buckets.erase(srv->buckets.begin() + i);
            break;
          }
        }
        rc = make_bucket(srv, q, &B);
      }
      if (rc == BRI17_ERR_BUSY) {
        ++it;
        continue;
      }
      if (rc == BRI17_ERR_OUT_OF_MEMORY || rc == BRI17_ERR_UNSUPPORTED_SIZE ||
          rc == BRI17_ERR_INVALID_ARGUMENT) {
        // The request cannot get a bucket: it fails alone; the requests in
        // flight are untouched (make_bucket released what it had built).
        cudaGetLastError();
        it = srv->queue.erase(it);
        progress = true;
        finish(srv, q, rc);
        continue;
      }
      if (rc != BRI17_OK) return rc;
    }
    const int z = B->in_flight ? -1 : free_slot(B);
    if (z < 0) {
      ++it;
      continue;
    }
    it = srv->queue.erase(it);
    progress = true;
    const int rc = admit(srv, B, z, q);
    if (rc != BRI17_OK) return rc;
  }
  // 3. Every idle bucket: a chunk if some slot's inner CG runs; the bucket
  //    stays in flight while any enqueued work (outer residuals,
  //    admissions, restarts) has not been retired.
  for (Bucket* B : srv->buckets) {
    if (B->in_flight) continue;
    if (bucket_has_inner(B)) {
      SRV_TRY(cudaGraphLaunch(B->graph, B->stream));
      B->enqueued = true;
    }
    if (B->enqueued) {
      B->in_flight = true;
      B->enqueued = false;
      progress = true;
    }
  }
  // 4. Nothing to do: wait a little for a chunk to complete.
  if (!progress) {
    const auto t_end = std::chrono::steady_clock::now() + std::chrono::microseconds(200);
    bool any = false;
    while (!any && std::chrono::steady_clock::now() < t_end) {
      for (Bucket* B : srv->buckets)
        if (B->in_flight && cudaStreamQuery(B->stream) != cudaErrorNotReady) any = true;
      for (Request* q : srv->finishing)
        if (cudaEventQuery(q->done_ev) != cudaErrorNotReady) any = true;
      if (!any) std::this_thread::sleep_for(std::chrono::microseconds(10));
    }
  }
  int n_active = 0;
  for (Bucket* B : srv->buckets)
    for (int z = 0; z < B->S; z++) n_active += B->slot_state[z] != kFree;
  if (active) *active = n_active;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "server step");
  return BRI17_OK;
}

extern "C" int bri17_server_poll(bri17_server* srv, bri17_request_result* out, int cap,
                                 int* count) {
  if (!srv || (!out && cap > 0) || !count) {
    set_error("null pointer");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  if (cap < 0) {
    set_error("cap must be >= 0");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  const int k = (int)std::min<size_t>(cap, srv->done.size());
  for (int i = 0; i < k; i++) out[i] = srv->done[i];
  srv->done.erase(srv->done.begin(), srv->done.begin() + k);
  *count = k;
  return BRI17_OK;
}

extern "C" double bri17_server_clock(const bri17_server* srv) {
  return srv ? srv->now() : 0.0;
}
