/*
 * bri17_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the bri17
 * matrix-free periodic finite-element stiffness operator.
 *
 * The reference library (sbrisard/bri17) is a header-only C++ template pair,
 * bri17::CartesianGrid<T,DIM> and bri17::Hooke<T,DIM>
 * (include/bri17/bri17.hpp:34-356), whose per-mode functions the user
 * combines with an FFT library; its only operator application is the test
 * harness StiffnessMatrixFactory::compute_Ku (tests/test_bri17.cpp:56-107).
 * This header exports, as plain C:
 *
 *   - an operator handle that owns one grid + one isotropic Hooke material
 *     (the state of bri17::Hooke, include/bri17/bri17.hpp:176-194),
 *   - batched forms of the per-mode functions Hooke::modal_stiffness and
 *     Hooke::modal_strain_displacement (:212-292) and of
 *     Hooke::modal_eigenstress_to_opposite_strain (:308-355),
 *   - the whole-field operator f = K u that compute_Ku computes,
 *   - the eigenstress right-hand side, the strain field u -> eps
 *     (compute_Bu, tests/test_bri17.cpp:194-245), and conjugate-gradient
 *     solvers of K u = b,
 *   - a continuous-batching solve server.
 *
 * Conventions.
 *   - Every function returns a status (bri17_status); none throws.
 *   - Fields use the reference's layout: structure of arrays, component c of
 *     node n at c * size + n, nodes row-major with the last axis fastest
 *     (include/bri17/bri17.hpp:78-93, tests/test_bri17.cpp:66-67).
 *   - Complex arrays are interleaved (re, im) pairs of the handle's scalar
 *     type (double for BRI17_F64, float for BRI17_F32).
 *   - "_dev" pointers are CUDA device pointers owned by the caller; work is
 *     enqueued on `stream` (a cudaStream_t, NULL = legacy default stream) and
 *     is stream-ordered: the call returns before the GPU finishes unless the
 *     function says otherwise.  "_host" pointers are host memory; those
 *     functions synchronise `stream` before returning.
 *   - A handle is externally synchronised (one thread at a time); distinct
 *     handles may be used concurrently.  A handle belongs to the CUDA device
 *     that was current when it was created: calls made with another device
 *     current return BRI17_ERR_INVALID_ARGUMENT.
 */
#ifndef BRI17_GB300_H_
#define BRI17_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bri17_status {
  BRI17_OK = 0,
  BRI17_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad dim, nu >= 0.5, ... */
  BRI17_ERR_UNSUPPORTED_SIZE = 2, /* an axis length the FFT plan rejects */
  BRI17_ERR_CUDA = 3,             /* a CUDA runtime call failed */
  BRI17_ERR_OUT_OF_MEMORY = 4,    /* device allocation failed */
  BRI17_ERR_NOT_CONVERGED = 5,    /* CG reached its iteration cap */
  BRI17_ERR_BREAKDOWN = 6,        /* NaN/Inf or non-positive curvature */
  BRI17_ERR_NO_DEVICE = 7,        /* no CUDA device visible */
  BRI17_ERR_BUSY = 8,             /* server full / request slot taken */
  BRI17_ERR_NOT_FOUND = 9,        /* unknown request id */
  BRI17_ERR_CANCELLED = 10,       /* request cancelled before it finished */
  BRI17_ERR_TIMEOUT = 11,         /* a bounded device wait ran out: results of
                                     the work it belonged to are invalid */
  BRI17_ERR_STAGNATED = 12        /* CG residual stopped decreasing above tol */
} bri17_status;

typedef enum bri17_precision {
  BRI17_F64 = 0, /* FP64 FFT, FP64 modal matvec */
  BRI17_F32 = 1  /* FP32 FFT, FP32 modal matvec */
} bri17_precision;

typedef struct bri17_op bri17_op; /* opaque operator handle */

/* Human-readable name of a status code (static storage).  No reference
 * counterpart: the reference returns no status and throws only from
 * unreachable branches (include/bri17/bri17.hpp:154-156). */
const char* bri17_status_string(int status);

/* Last CUDA / validation message recorded by this thread (static storage per
 * thread; empty string if none).  No reference counterpart. */
const char* bri17_last_error(void);

/* Library version string, e.g. "0.1.0" (the reference is v0.1,
 * metadata/version.txt:1). */
const char* bri17_version(void);

/*
 * Create an operator for the grid shape[0] x ... x shape[dim-1] of box size
 * L[0..dim-1] and the isotropic Hooke material (mu, nu).
 * Replaces: bri17::CartesianGrid<T,DIM>(shape, L) +
 * bri17::Hooke<T,DIM>(mu, nu, grid)   (include/bri17/bri17.hpp:54-58, :193-194)
 * plus the FFTW plan set-up of StiffnessMatrixFactory
 * (tests/test_bri17.cpp:110-128).
 * dim is 2 or 3; every shape[i] >= 1 and <= 1024 with prime factors <= 61;
 * L[i] > 0; mu > 0; -1 < nu < 0.5.  Allocates the device work space on the
 * current CUDA device.
 */
int bri17_op_create(int dim, const int* shape, const double* L, double mu,
                    double nu, int precision, bri17_op** op);

/* Release a handle and its device memory (NULL is accepted).  Replaces the
 * end of life of the bri17::Hooke value and of the FFT buffers
 * (~FFTWComplexBuffer, tests/test_bri17.cpp:40). */
int bri17_op_destroy(bri17_op* op);

/* Grid size |N| (number of nodes = cells; CartesianGrid::size,
 * include/bri17/bri17.hpp:54-58) and device work-space bytes. */
int bri17_op_info(const bri17_op* op, int64_t* size, int64_t* workspace_bytes);

/*
 * Per-pass timing (diagnostics; no reference counterpart).  While enabled,
 * each operator application on this handle records CUDA events around each
 * of its kernel launches, on the launch stream.  bri17_op_pass_times
 * synchronises those events and returns, per pass id, the summed device time
 * in ms and the number of launches since the previous call, then resets.
 * Pass ids: 0 rows_r2c, 1 axis1 forward, 2 axis0 fused, 3 axis1 inverse,
 * 4 rows_c2r (2D handles have no axis-1 passes).
 */
int bri17_op_set_pass_timing(bri17_op* op, int enable);
int bri17_op_pass_times(bri17_op* op, double* ms, int64_t* launches,
                        int max_passes, int* npasses);
const char* bri17_pass_name(int pass);

/* Change the material of an existing handle (no reallocation).  Replaces
 * constructing a new bri17::Hooke(mu, nu, grid) on the same grid
 * (include/bri17/bri17.hpp:193-194); same bounds as bri17_op_create. */
int bri17_op_set_material(bri17_op* op, double mu, double nu);

/*
 * Form of the fused axis-0 stiffness pass (diagnostics; no reference
 * counterpart): 0 register-resident, 1 shared-memory staged, 2 TMA-staged
 * (tensor copies of whole tiles; FP32, 3D, even shape[1]), 3 TMA-staged with
 * the spectra kept in registers between the transforms (float-pair
 * handles: 1 or 2, other values select 1).  FP32 handles with a
 * power-of-two first axis pick the fastest by timing at creation; a first
 * axis of length 3 * 2^k (24..192) always takes the staged form.  A form
 * that does not apply to the handle's grid falls back to the next
 * applicable one at launch.  Results agree between forms to rounding.
 */
int bri17_op_fused_form(const bri17_op* op, int* form);
int bri17_op_set_fused_form(bri17_op* op, int form);

/*
 * Float-pair arithmetic (no reference counterpart): on an FP64 handle,
 * bri17_apply_stiffness and bri17_apply_stiffness_host compute in pairs of
 * floats (hi + lo, 48-bit significands, error-free transformations on the
 * FP32 pipe, which GB300 runs at about 60x its FP64 rate) with FP64 fields
 * in memory.  Relative error against the FP64 operator is about 1e-14,
 * within the 1e-12 parity bound of the FP64 path.  Values keep their 48 bits
 * for magnitudes 1e-30..1e37.  Power-of-two grids, 2D or 3D: the strided
 * axes (shape[0], and shape[1] in 3D) in 64..512, the last axis in
 * 128..1024 (else BRI17_ERR_UNSUPPORTED_SIZE).  The plain CG solver's
 * operator applications on the handle run in float pairs too (the mixed
 * solvers' FP64 residuals use them on such grids either way: see
 * bri17_cg_solve); strain, right-hand side and the per-mode batches stay in
 * FP64.  Off by default.
 */
int bri17_op_set_float_pair(bri17_op* op, int enable);

/*
 * Bounded device-side waits (tensor-copy completions) that ran out on the
 * current device since the previous call; 0 in normal operation.  A nonzero
 * count means some operator results of that period are invalid.
 * Diagnostics; no reference counterpart.
 */
int bri17_wait_timeouts(int* count);

/*
 * Failure of a bounded device wait, reported per handle (no reference
 * counterpart).  The kernels that stage tiles by tensor copies (the FP32
 * and float-pair axis-0 passes) wait for those copies at most one second;
 * a wait that runs out, or a tile whose shared-memory window is misplaced,
 * leaves that tile untransformed -- the output of that call is invalid --
 * and sets the handle's status.  Stream-ordered calls return before their
 * kernels run, so the failure reaches the caller as BRI17_ERR_TIMEOUT from:
 *   - bri17_op_sync_status, which synchronises `stream` first;
 *   - the synchronous entry points (bri17_apply_stiffness_host,
 *     bri17_cg_solve) for their own work;
 *   - the next field entry point called on the handle (apply_stiffness,
 *     apply_stiffness_host, apply_strain, eigenstress_rhs,
 *     eigenstress_to_opposite_strain, cg_solve), which then enqueues
 *     nothing.
 * Each failure is reported once; the handle stays usable.
 */
int bri17_op_sync_status(bri17_op* op, void* stream);

/*
 * Diagnostics (no reference counterpart): the limit, in nanoseconds of GPU
 * global time, of the first wait on tile copies in the tensor-copy kernels
 * on the current device; 0 makes every such wait give up at once (for
 * testing the failure path).  Default 1e9 (one second).  A CTA whose wait
 * gives up still waits, with the default limit, for its own copies to land
 * before it leaves.
 */
int bri17_set_wait_limit_ns(uint64_t ns);

/*
 * Batched Hooke::modal_stiffness (include/bri17/bri17.hpp:247-292; exported
 * to Python as Hooke*f64.modal_stiffness_matrix, python/pybri17.cpp:82-87).
 * k_dev: n x dim int32 multi-indices; K_dev: n x dim x dim complex (row-major
 * per mode).  For 0 <= k[i] < shape[i] the values equal the reference's bit
 * for bit; other k are reduced modulo shape[i] first.
 */
int bri17_modal_stiffness_batch(const bri17_op* op, const int* k_dev,
                                int64_t n, void* K_dev, void* stream);

/*
 * Batched Hooke::modal_strain_displacement (include/bri17/bri17.hpp:212-236,
 * python/pybri17.cpp:76-81).  B_dev: n x dim complex.
 */
int bri17_modal_strain_displacement_batch(const bri17_op* op, const int* k_dev,
                                          int64_t n, void* B_dev,
                                          void* stream);

/*
 * Batched Hooke::modal_eigenstress_to_opposite_strain
 * (include/bri17/bri17.hpp:308-355, python/pybri17.cpp:88-95).
 * tau_dev: n x sym complex Mandel components (sym = 3 in 2D, 6 in 3D, order
 * xx,yy[,zz],[yz,zx,]xy with sqrt(2) on the shears); eta_dev: n x sym complex.
 * k = 0 gives 0, as in the reference.
 */
int bri17_modal_eigenstress_to_opposite_strain_batch(const bri17_op* op,
                                                     const int* k_dev,
                                                     int64_t n,
                                                     const void* tau_dev,
                                                     void* eta_dev,
                                                     void* stream);

/*
 * The three per-mode functions on host buffers, for code written against
 * the reference's per-mode calls (include/bri17/bri17.hpp:212-355, called
 * mode by mode from python/demo.py:34-40 and tests/test_bri17.cpp:63-91):
 * k (n x dim int32), tau, K, B and eta are host memory in the layouts of
 * the _batch functions above, with the same values (K bit for bit).  Each
 * call copies its inputs into page-locked staging that the handle keeps
 * (mapped into the device), runs one kernel on a private stream of the
 * handle, waits for it and copies the result out: no device allocation
 * after the first call of a size, and the caller's streams are not
 * touched.  Synchronous; calls on one handle may come from several threads
 * (they are serialised).  A call costs a kernel launch plus a
 * synchronisation -- microseconds -- so batches of many modes amortise it.
 */
int bri17_modal_stiffness_host(const bri17_op* op, const int* k, int64_t n, void* K);
int bri17_modal_strain_displacement_host(const bri17_op* op, const int* k, int64_t n,
                                         void* B);
int bri17_modal_eigenstress_to_opposite_strain_host(const bri17_op* op, const int* k,
                                                    int64_t n, const void* tau, void* eta);

/*
 * f = K u: the periodic stiffness operator, computed as
 * f = (|h|/|N|) IDFT(K(k) DFT(u)(k)), i.e. StiffnessMatrixFactory::compute_Ku
 * (tests/test_bri17.cpp:56-107), on real fields.  u_dev and f_dev are
 * dim x size real arrays of the handle's scalar type; they may alias.
 */
int bri17_apply_stiffness(bri17_op* op, const void* u_dev, void* f_dev,
                          void* stream);

/*
 * f = K u without any device allocation (FP64).  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory -- a
 * plugin whose host application owns every device allocation and forbids
 * cudaMalloc, code held to a device-memory budget fixed in advance, or a
 * caller that must not let cudaMalloc/cudaFree synchronise the device.
 * The caller passes the grid, the material, u_dev and f_dev (dim x size FP64
 * device arrays, SoA, as bri17_apply_stiffness); results equal
 * bri17_apply_stiffness's to rounding (within 1e-12 relative).
 * Scratch (per-axis tables + the FP64 half spectrum) lives in one fixed
 * 64 MiB device array that every GPU loading this library holds until the
 * process exits; grids needing more (tables + dim * n0 * n1 * (n2/2+1) * 16
 * bytes, e.g. anything above 128^3) return BRI17_ERR_UNSUPPORTED_SIZE.
 * The tables are written into that array by a kernel on `stream`, so the
 * call copies nothing from the host and is stream-ordered like
 * bri17_apply_stiffness.  The first call on a device looks up that array's
 * device address on that device (set-up), so make the first call before
 * any stream capture.  Every call shares the one array and rewrites all of
 * it that it reads (nothing needs to start at zero); calls whose GPU work
 * overlaps -- on different streams, or from different threads -- race on it
 * and must be serialised by the caller.
 */
int bri17_apply_stiffness_noalloc(int dim, const int* shape, const double* L,
                                  double mu, double nu, const double* u_dev,
                                  double* f_dev, void* stream);

/*
 * Same operator with host buffers; synchronises `stream` before returning.
 * Replaces compute_Ku called on host data (tests/test_bri17.cpp:56-107), the
 * form a binding that owns numpy arrays would call.  Page-locked buffers (cudaHostAlloc / cudaHostRegister) are read and written
 * in place by the first and last passes over the host link; other host
 * memory goes through device staging buffers with the copies pipelined per
 * component against the passes.
 */
int bri17_apply_stiffness_host(bri17_op* op, const void* u_host, void* f_host,
                               void* stream);

/*
 * eps = B u: cell-averaged strains (Mandel, sym components) of nodal
 * displacements, StrainDisplacementMatrixFactory::compute_Bu
 * (tests/test_bri17.cpp:194-245).  eps_dev: sym x size real.
 */
int bri17_apply_strain(bri17_op* op, const void* u_dev, void* eps_dev,
                       void* stream);

/*
 * Nodal forces of a cell-wise eigenstress: b = -|h| B^T tau, computed in
 * Fourier space as b_hat = -|h| tau_hat . conj(B(k)) (the right-hand side of
 * include/bri17/bri17.hpp:340).  tau_dev: sym x size real (Mandel);
 * b_dev: dim x size real.  b has zero mean.
 */
int bri17_eigenstress_rhs(bri17_op* op, const void* tau_dev, void* b_dev,
                          void* stream);

/*
 * Opposite strain eta = -eps of a cell-wise eigenstress field tau: the
 * whole-field form of Hooke::modal_eigenstress_to_opposite_strain
 * (include/bri17/bri17.hpp:308-355) as python/demo.py:24-40 applies it mode
 * by mode: eta = ifft(eta_hat(fft(tau))), eta_hat(k) = sym(B (x) K^-1
 * (tau_hat . conj(B))) in Mandel form, eta_hat(0) = 0.  The direct
 * (per-mode) solution of the eigenstress problem.  tau_dev, eta_dev:
 * sym x size, the handle's precision (sym = 3 in 2D, 6 in 3D).
 */
int bri17_eigenstress_to_opposite_strain(bri17_op* op, const void* tau_dev,
                                         void* eta_dev, void* stream);

/* Conjugate-gradient modes. */
typedef enum bri17_cg_mode {
  BRI17_CG_PLAIN = 0,        /* CG in the handle's precision */
  BRI17_CG_MIXED = 1,        /* FP32 CG with FP64 reliable updates: the FP32
                                correction is folded into the FP64 iterate and
                                the residual recomputed in FP64 (r = b - K x,
                                zero-mean projection) each time it has dropped
                                10x; the search direction is kept */
  BRI17_CG_MIXED_RESTART = 2 /* classic iterative refinement: FP32 CG restarted
                                on each FP64 residual */
} bri17_cg_mode;

typedef struct bri17_cg_info {
  int iterations;        /* total operator applications inside CG */
  int outer_iterations;  /* FP64 residual recomputations (mixed modes), else 1 */
  double rel_residual;   /* final ||b - K x|| / ||b|| (FP64, recomputed) */
  int status;            /* bri17_status of the solve */
} bri17_cg_info;

/*
 * No reference counterpart as an iterative solver: the reference solves the
 * eigenstress problem mode by mode (python/demo.py:24-40 over
 * Hooke::modal_eigenstress_to_opposite_strain, include/bri17/bri17.hpp:308-355),
 * which is this library's oracle for it.
 * Solve K x = b by conjugate gradients, to ||b - K x|| <= tol ||b||, with x
 * projected to zero mean per component (the null space of K is the rigid
 * translations, sphinx/theory.rst eq. (17) note).  b_dev and x_dev are FP64
 * (dim x size).  On entry x_dev is the initial guess (zero it for a cold
 * start).  BRI17_CG_MIXED needs an FP64 handle; it builds an FP32 twin
 * internally on first use.  The mixed modes compute their FP64 residuals
 * (r = b - K x) in float pairs (see bri17_op_set_float_pair; about 1e-14
 * from the FP64 operator) whenever the grid has float-pair instances, with
 * float pairs on the handle or not; BRI17_MIXED_RESIDUAL=f64 in the
 * environment keeps them on the FP64 pipe.  The plain solver on an FP64
 * handle stays on the FP64 pipe unless float pairs are on; it recomputes
 * the true residual at every 100x drop of the recursive one (and at least
 * every 256 iterations) and, when that stops decreasing above tol, returns
 * BRI17_ERR_STAGNATED with the iterate of smallest true residual in x_dev.
 * Synchronises `stream` (the stopping test reads the residual).
 */
int bri17_cg_solve(bri17_op* op, const double* b_dev, double* x_dev,
                   double tol, int max_iterations, int mode,
                   bri17_cg_info* info, void* stream);

/*
 * Serving (no reference counterpart): a continuous-batching solve server on
 * the current device.
 * Requests (3D eigenstress problems of any supported grid and material) are
 * admitted while their device footprint fits in `memory_budget_bytes`,
 * solved concurrently in mixed precision, and retired when converged.
 */
typedef struct bri17_server bri17_server;

typedef struct bri17_request_result {
  int64_t id;
  int status;             /* bri17_status */
  int iterations;
  int outer_iterations;
  double rel_residual;
  double submit_time_s;   /* server clock at submit / admit / finish */
  double admit_time_s;
  double finish_time_s;
} bri17_request_result;

/*
 * Create / destroy a server (no reference counterpart).
 * max_active (1..256): most request slots per bucket (one bucket per grid
 * geometry).  A bucket gets enough slots for about 48 M unknowns of batched
 * work per iteration, at least 8, at most max_active.
 */
int bri17_server_create(int64_t memory_budget_bytes, int max_active,
                        bri17_server** srv);
int bri17_server_destroy(bri17_server* srv);

/*
 * Scheduling policy (no reference counterpart) for buckets created from now on: 0 (default) all
 * streams equal, highest throughput; 1 smaller geometries on higher-priority
 * streams, so small requests are not queued behind large buckets' kernels
 * (on the 512-request benchmark stream: p50 latency 2.4 -> 0.5 s,
 * throughput 51 -> 44 solves/s).
 */
int bri17_server_set_size_priority(bri17_server* srv, int enable);

/*
 * Submit one eigenstress solve (no reference counterpart; the reference
 * solves it mode by mode, python/demo.py:24-40).  tau_host: 6 x size FP64 Mandel eigenstress
 * (copied at submit); the server owns the request until bri17_server_poll
 * returns it.  x_host: dim x size FP64, written with the solution when the
 * request finishes (must stay valid until then).  Returns the request id in
 * *id.
 */
int bri17_server_submit(bri17_server* srv, const int* shape, const double* L,
                        double mu, double nu, const double* tau_host,
                        double* x_host, double tol, int max_iterations,
                        int64_t* id);

/*
 * Same (no reference counterpart), without the copy of tau at submit: tau_host is read when the request
 * is admitted and must stay valid and unchanged until bri17_server_poll
 * returns the request.  With page-locked tau_host and x_host (cudaHostAlloc,
 * cudaHostRegister) the upload and the solution's download are asynchronous
 * copies, so admissions and retirements never block the server's step.
 * (bri17_server_submit also downloads asynchronously into a page-locked
 * x_host.)
 */
int bri17_server_submit_borrowed(bri17_server* srv, const int* shape,
                                 const double* L, double mu, double nu,
                                 const double* tau_host, double* x_host,
                                 double tol, int max_iterations, int64_t* id);

/* Advance the server: admit, run one scheduling quantum, retire.  Returns
 * the number of active requests in *active.  No reference counterpart. */
int bri17_server_step(bri17_server* srv, int* active);

/* Pop up to `cap` (>= 0) finished results; *count receives how many.  No
 * reference counterpart. */
int bri17_server_poll(bri17_server* srv, bri17_request_result* out, int cap,
                      int* count);

/*
 * Fault injection (diagnostics; no reference counterpart): the next bucket
 * creation of this server fails at the allocation of its work buffer
 * number `at` (0-based; the buffers allocated before it are released) as
 * cudaMalloc does when device memory runs out; -1 cancels.  A request that
 * cannot get a bucket -- injected or real out-of-memory, or a grid the
 * operator rejects -- finishes alone with that status
 * (BRI17_ERR_OUT_OF_MEMORY, ...); requests already in flight are not
 * affected.
 */
int bri17_server_inject_alloc_failure(bri17_server* srv, int at);

/* Cancel a queued or running request (its result reports CANCELLED).  No
 * reference counterpart. */
int bri17_server_cancel(bri17_server* srv, int64_t id);

/* Server clock (seconds since creation).  No reference counterpart. */
double bri17_server_clock(const bri17_server* srv);

#ifdef __cplusplus
}
#endif

#endif /* BRI17_GB300_H_ */
