// operator.cu -- operator handle, FFT plans, per-mode batch kernels and the
// C ABI of the periodic stiffness operator (include/bri17_gb300.h).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include <cudaTypedefs.h>

#include "op.cuh"
#include "passes.cuh"
#include "passes_p2.cuh"

// The float-pair operator (defined with its C ABI below).
static int run_stiffness_df(bri17_op* op, const double* u, double* f, int form,
                            cudaStream_t st, const bri17gb::df64* mat = nullptr);

namespace bri17gb {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? BRI17_ERR_OUT_OF_MEMORY
                                        : BRI17_ERR_CUDA;
}

static int invalid(const char* msg) {
  set_error(msg);
  return BRI17_ERR_INVALID_ARGUMENT;
}

// A handle's device memory lives on the device that was current when it was
// created; calls must be made with that device current.
int check_device(const bri17_op* op) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != op->device) {
    set_error("the current CUDA device differs from the handle's device");
    return BRI17_ERR_INVALID_ARGUMENT;
  }
  return BRI17_OK;
}

int take_status(bri17_op* op) {
  int rc = BRI17_OK;
  for (bri17_op* o : {op, op->twin32}) {
    if (!o || !o->status_host) continue;
    // Host atomics: a kernel's store that lands after the exchange is kept
    // for the next check.
    const int timeout = __atomic_exchange_n(&o->status_host[0], 0, __ATOMIC_SEQ_CST);
    const int skipped = __atomic_exchange_n(&o->status_host[1], 0, __ATOMIC_SEQ_CST);
    if (timeout || skipped) {
      set_error(timeout ? "a bounded device wait on tile copies ran out: the output of the "
                          "operator work it belonged to is invalid"
                        : "a tile was skipped (misplaced shared-memory window): the output of "
                          "the operator work it belonged to is invalid");
      rc = BRI17_ERR_TIMEOUT;
    }
  }
  return rc;
}

// ---------------------------------------------------------------------------
// Plans.

bool make_plan(int n, AxisPlan* p) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  if (n < 1) return false;
  int e = 0, m = n;
  while (m % 2 == 0) {
    m /= 2;
    e++;
  }
  std::vector<int> r;
  const int q = e / 4, rem = e % 4;
  for (int i = 0; i < q; i++) r.push_back(16);
  if (rem == 1) {
    if (q >= 1) {
      r.pop_back();
      r.push_back(8);
      r.push_back(4);
    } else {
      r.push_back(2);
    }
  } else if (rem == 2) {
    r.push_back(4);
  } else if (rem == 3) {
    r.push_back(8);
  }
  for (int f = 3; m > 1; f += 2) {
    while (m % f == 0) {
      if (f > kMaxGenericRadix) return false;
      r.push_back(f);
      m /= f;
    }
  }
  if ((int)r.size() > kMaxStages) return false;
  p->nstages = (int)r.size();
  for (int i = 0; i < p->nstages; i++) p->radix[i] = r[i];
  return true;
}

// ---------------------------------------------------------------------------
// Tables.  Twiddles are computed in long double with an exact argument and
// rounded once; the modal factors repeat the reference's double expressions
// (include/bri17/bri17.hpp:217-222, :258-264) so that the per-mode API is
// bit-identical to it.

constexpr double kPi = 3.141592653589793238462643383279502884;

struct HostTables {
  std::vector<double> twr, twi, kphi, kchi, kpsi, bc, bs, ec, es;
};

static void host_tables(int n, double L, HostTables* t) {
  const long double pil = 3.141592653589793238462643383279502884L;
  t->twr.resize(n);
  t->twi.resize(n);
  t->kphi.resize(n);
  t->kchi.resize(n);
  t->kpsi.resize(n);
  t->bc.resize(n);
  t->bs.resize(n);
  t->ec.resize(n);
  t->es.resize(n);
  for (int k = 0; k < n; k++) {
    const long double ang = 2.0L * pil * (long double)k / (long double)n;
    t->twr[k] = (double)cosl(ang);
    t->twi[k] = (double)-sinl(ang);
    const double h = L / n;
    const double beta = 2 * kPi * k / n;
    t->kphi[k] = 2 * (1 - cos(beta)) / h / h;
    t->kchi[k] = (2 + cos(beta)) / 3;
    t->kpsi[k] = sin(beta) / h;
    const double alpha = kPi * k / n;
    t->bc[k] = cos(alpha);
    t->bs[k] = sin(alpha) * n / L;
    t->ec[k] = cos(alpha);
    t->es[k] = sin(alpha);
  }
}

static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <typename T>
static void fill_tables(const std::vector<HostTables>& ht, const int* n,
                        int dim, unsigned char* host, size_t* off,
                        Tables<T>* tab, unsigned char* dev) {
  for (int i = 0; i < 3; i++) {
    tab->tw[i] = nullptr;
    tab->kphi[i] = tab->kchi[i] = tab->kpsi[i] = tab->bc[i] = tab->bs[i] =
        nullptr;
    tab->ea[i] = nullptr;
  }
  for (int i = 0; i < dim; i++) {
    const HostTables& t = ht[i];
    const int m = n[i];
    // twiddles
    {
      cplx<T>* h = reinterpret_cast<cplx<T>*>(host + *off);
      for (int k = 0; k < m; k++) {
        h[k].x = (T)t.twr[k];
        h[k].y = (T)t.twi[k];
      }
      tab->tw[i] = reinterpret_cast<const cplx<T>*>(dev + *off);
      *off = align16(*off + m * sizeof(cplx<T>));
    }
    {
      cplx<T>* h = reinterpret_cast<cplx<T>*>(host + *off);
      for (int k = 0; k < m; k++) {
        h[k].x = (T)t.ec[k];
        h[k].y = (T)t.es[k];
      }
      tab->ea[i] = reinterpret_cast<const cplx<T>*>(dev + *off);
      *off = align16(*off + m * sizeof(cplx<T>));
    }
    const std::vector<double>* src[5] = {&t.kphi, &t.kchi, &t.kpsi, &t.bc,
                                         &t.bs};
    const T** dst[5] = {&tab->kphi[i], &tab->kchi[i], &tab->kpsi[i],
                        &tab->bc[i], &tab->bs[i]};
    for (int j = 0; j < 5; j++) {
      T* h = reinterpret_cast<T*>(host + *off);
      for (int k = 0; k < m; k++) h[k] = (T)(*src[j])[k];
      *dst[j] = reinterpret_cast<const T*>(dev + *off);
      *off = align16(*off + m * sizeof(T));
    }
  }
}

static size_t tables_bytes(const int* n, int dim, size_t tsize) {
  size_t b = 0;
  for (int i = 0; i < dim; i++) {
    b = align16(b + n[i] * 2 * tsize);
    b = align16(b + n[i] * 2 * tsize);
    for (int j = 0; j < 5; j++) b = align16(b + n[i] * tsize);
  }
  return b;
}

// ---------------------------------------------------------------------------
// Launch helpers.

constexpr int kTileElems = 2048;        // complex values per CTA tile
constexpr size_t kFusedSmemBudget = 100 * 1024;
constexpr size_t kMaxSmem = 227 * 1024;

template <typename T>
static void set_smem_attrs() {
  static std::atomic<unsigned long long> done{0};
  once_per_device(&done, [] {
    cudaFuncSetAttribute(rows_r2c<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(rows_c2r<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis_c2c<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis_c2c<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(rows_r2c_p2<T, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(rows_c2r_p2<T, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis_c2c_p2<T, false, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis_c2c_p2<T, true, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis0_stiffness_p2<T, 2, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    cudaFuncSetAttribute(axis0_stiffness_p2<T, 3, RtEng>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    ct_set_smem_attrs(kMaxSmem);
    if constexpr (!std::is_same<T, df64>::value) ct3_set_smem_attrs_t<T>(kMaxSmem);
#define SET_FUSED(D, M) \
  cudaFuncSetAttribute(axis0_fused<T, D, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem)
    SET_FUSED(2, kModeStiffness);
    SET_FUSED(3, kModeStiffness);
    SET_FUSED(2, kModeStrain);
    SET_FUSED(3, kModeStrain);
    SET_FUSED(2, kModeRhs);
    SET_FUSED(3, kModeRhs);
    SET_FUSED(2, kModeSolve);
    SET_FUSED(3, kModeSolve);
#undef SET_FUSED
    cudaGetLastError();
  });
}

// Rows per CTA for the last-axis passes: about kTileElems complex values,
// and, when a batch mask is in use, a divisor of the rows of one entry so
// that no CTA straddles two entries.
static int rows_per_cta(int m, int64_t nrows, int64_t rows_per_entry, bool masked) {
  int64_t r = std::max<int64_t>(1, std::min<int64_t>(nrows, kTileElems / m));
  if (masked) {
    while (r > 1 && rows_per_entry % r != 0) r--;
  }
  return (int)r;
}

// Rows per CTA of the register-resident row passes: 256 threads' worth,
// a power of two dividing the rows of one batch entry when masked.
static int rows_p8(int T, int64_t nrows, int64_t unit, bool masked) {
  int rb = kP2Threads / T;
  if (masked)
    while (rb > 1 && unit % rb != 0) rb /= 2;
  return (int)std::max<int64_t>(1, std::min<int64_t>(rb, nrows));
}

template <typename T>
static int launch_rows_r2c(const Geometry& g, const T* x, cplx<T>* X,
                           int64_t nrows, const Tables<T>& tab, BatchMask mask,
                           cudaStream_t st) {
  if (g.use_ct3_row && ct3_rows_r2c<T>(g.n[g.dim - 1] / 2, x, X, nrows, g.H,
                                       tab.tw[g.dim - 1], mask, st))
    return BRI17_OK;
  if (g.use_p8_row) {
    const Plan8& p = g.p8_row;
    if (ct_rows_r2c<T>(p.n, x, X, nrows, g.H, tab.tw[g.dim - 1], mask, st)) return BRI17_OK;
    const int rb = rows_p8(p.T, nrows, mask.unit, mask.flags != nullptr);
    const int pitch = exchange_pitch(p.n, rb, (int)sizeof(cplx<T>), false);
    const size_t smem = (3 * p.n + 1 + (size_t)rb * pitch) * sizeof(cplx<T>);
    launch_pdl(rows_r2c_p2<T, RtEng>, (unsigned)((nrows + rb - 1) / rb), p.T * rb, smem, st,
               x, X, nrows, g.H, RtEng{p}, tab.tw[g.dim - 1], rb, pitch, mask);
    return BRI17_OK;
  }
  const int n = g.n[g.dim - 1];
  const int m = (n % 2 == 0) ? n / 2 : n;
  const int pitch = m + 1;
  const int rows = rows_per_cta(m, nrows, mask.unit, mask.flags != nullptr);
  size_t smem = n * sizeof(cplx<T>) + 2 * (size_t)rows * pitch * sizeof(cplx<T>);
  const int64_t grid = (nrows + rows - 1) / rows;
  launch_pdl(rows_r2c<T>, (unsigned)grid, kThreads, smem, st, x, X, nrows, n, g.H, g.plan_row,
                                                      tab.tw[g.dim - 1], rows, pitch, mask);
  return BRI17_OK;
}

template <typename T>
static int launch_rows_c2r(const Geometry& g, const cplx<T>* X, T* x,
                           int64_t nrows, const Tables<T>& tab, BatchMask mask,
                           cudaStream_t st) {
  if (g.use_ct3_row && ct3_rows_c2r<T>(g.n[g.dim - 1] / 2, X, x, nrows, g.H,
                                       tab.tw[g.dim - 1], mask, st))
    return BRI17_OK;
  if (g.use_p8_row) {
    const Plan8& p = g.p8_row;
    if (ct_rows_c2r<T>(p.n, X, x, nrows, g.H, tab.tw[g.dim - 1], mask, st)) return BRI17_OK;
    const int rb = rows_p8(p.T, nrows, mask.unit, mask.flags != nullptr);
    const int pitch = exchange_pitch(p.n, rb, (int)sizeof(cplx<T>), false);
    const size_t smem = (2 * p.n + (size_t)rb * pitch) * sizeof(cplx<T>);
    launch_pdl(rows_c2r_p2<T, RtEng>, (unsigned)((nrows + rb - 1) / rb), p.T * rb, smem, st,
               X, x, nrows, g.H, RtEng{p}, tab.tw[g.dim - 1], rb, pitch, mask);
    return BRI17_OK;
  }
  const int n = g.n[g.dim - 1];
  const int m = (n % 2 == 0) ? n / 2 : n;
  const int pitch = m + 1;
  const int rows = rows_per_cta(m, nrows, mask.unit, mask.flags != nullptr);
  size_t smem = n * sizeof(cplx<T>) + 2 * (size_t)rows * pitch * sizeof(cplx<T>);
  const int64_t grid = (nrows + rows - 1) / rows;
  launch_pdl(rows_c2r<T>, (unsigned)grid, kThreads, smem, st, X, x, nrows, n, g.H, g.plan_row,
                                                      tab.tw[g.dim - 1], rows, pitch, mask);
  return BRI17_OK;
}

namespace {

// Wavefronts of one warp-wide shared-memory access: the largest number of
// distinct 4-byte words any of the 32 banks serves.
int access_wavefronts(const int* byte_addr, int lanes, int csize) {
  int words[128];
  int nw = 0;
  for (int l = 0; l < lanes; l++)
    for (int w = 0; w < csize / 4; w++) words[nw++] = byte_addr[l] / 4 + w;
  int best = 0;
  for (int b = 0; b < 32; b++) {
    int distinct = 0;
    for (int i = 0; i < nw; i++) {
      if (words[i] % 32 != b) continue;
      bool seen = false;
      for (int k = 0; k < i && !seen; k++) seen = words[k] == words[i];
      if (!seen) distinct++;
    }
    best = std::max(best, distinct);
  }
  return best;
}

// Stage schedule of the engines: E = 8 as make_plan8 (8s, then 4 x 4 or
// 4); E = 16 as the compile-time engine's (16s, then one stage of the
// remaining power of two); E = 12 for 3 * 2^k (4s, a 2, the 3 last).
struct StagePlan {
  int T, nst, radix[12];
};

bool stage_plan(int n, int E, StagePlan* sp) {
  if (E == 8) {
    Plan8 p;
    if (!make_plan8(n, &p)) return false;
    sp->T = p.T;
    sp->nst = p.nst;
    for (int s = 0; s < p.nst; s++) sp->radix[s] = p.radix[s];
    return true;
  }
  if (E == 12) {
    // PE3: radix 4s, one 2 when log2(n / 3) is odd, the 3 last.
    if (!is_3pow2(n) || n > 768) return false;
    int lp = 0;
    while ((1 << lp) < n / 3) lp++;
    sp->T = n / 12;
    sp->nst = 0;
    for (int s = 0; s < lp / 2; s++) sp->radix[sp->nst++] = 4;
    if (lp % 2) sp->radix[sp->nst++] = 2;
    sp->radix[sp->nst++] = 3;
    return true;
  }
  if (E != 16 || !is_pow2(n) || n < 16 || n > 1024) return false;
  int ln = 0;
  while ((1 << ln) < n) ln++;
  sp->T = n / 16;
  sp->nst = 0;
  for (int s = 0; s < ln / 4; s++) sp->radix[sp->nst++] = 16;
  if (ln % 4) sp->radix[sp->nst++] = 1 << (ln % 4);
  return true;
}

long exchange_wavefronts(const StagePlan& p, int E, int lines, int pitch, int csize,
                         bool lines_fastest) {
  const int T = p.T;
  const int nthreads = T * lines;
  long total = 0;
  int addr[32];
  auto pad = [](int q) { return q + (q >> 4); };
  for (int w0 = 0; w0 < nthreads; w0 += 32) {
    const int lanes = std::min(32, nthreads - w0);
    int Ns = 1;
    for (int s = 0; s + 1 < p.nst; s++) {
      const int R = p.radix[s], M = E / R;
      for (int m = 0; m < M; m++)
        for (int r = 0; r < R; r++) {
          for (int l = 0; l < lanes; l++) {
            const int tid = w0 + l;
            const int line = lines_fastest ? tid % lines : tid / T;
            const int t = lines_fastest ? tid / lines : tid % T;
            const int j = t + T * m, jm = j & (Ns - 1);
            addr[l] = (line * pitch + pad((j - jm) * R + jm + r * Ns)) * csize;
          }
          total += access_wavefronts(addr, lanes, csize);
        }
      for (int q = 0; q < E; q++) {
        for (int l = 0; l < lanes; l++) {
          const int tid = w0 + l;
          const int line = lines_fastest ? tid % lines : tid / T;
          const int t = lines_fastest ? tid / lines : tid % T;
          addr[l] = (line * pitch + pad(t + T * q)) * csize;
        }
        total += access_wavefronts(addr, lanes, csize);
      }
      Ns *= R;
    }
  }
  return total;
}

}  // namespace

int exchange_pitch(int n, int lines, int csize, bool lines_fastest, int E) {
  static std::mutex mu;
  static std::map<long, int> cache;
  const long key =
      ((((long)n * 4096 + lines) * 64 + csize) * 2 + (lines_fastest ? 1 : 0)) * 32 + E;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  StagePlan p;
  int best = pitch8(n);
  if (stage_plan(n, E, &p) && lines >= 1) {
    long best_w = -1;
    for (int d = 0; d < 16; d++) {
      const int pitch = n + n / 16 + d;
      const long w = exchange_wavefronts(p, E, lines, pitch, csize, lines_fastest);
      if (best_w < 0 || w < best_w) {
        best_w = w;
        best = pitch;
      }
    }
  }
  cache[key] = best;
  return best;
}

bool encode_tiled_map_3d(CUtensorMap* map, const void* base, int elem_bytes, uint64_t dim0,
                         uint64_t dim1, uint64_t dim2, uint64_t stride1_bytes,
                         uint64_t stride2_bytes, uint32_t box0, uint32_t box1) {
  // cuTensorMapEncodeTiled through the runtime's driver entry point (no
  // link-time dependency on the driver library).
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      fn = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode || (elem_bytes != 4 && elem_bytes != 8)) return false;
  const cuuint64_t dims[3] = {dim0, dim1, dim2};
  const cuuint64_t strides[2] = {stride1_bytes, stride2_bytes};
  const cuuint32_t box[3] = {box0, box1, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(
      map, elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
      3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <typename T, bool INV>
static int launch_axis1(const Geometry& g, cplx<T>* X, int64_t nouter,
                        const Tables<T>& tab, BatchMask mask, cudaStream_t st) {
  if (g.use_ct3[1] && ct3_axis_c2c<T, INV>(g.n[1], X, g.H, nouter, tab.tw[1], mask, st))
    return BRI17_OK;
  if (g.use_p8[1]) {
    const Plan8& p = g.p8[1];
    if (ct_axis_c2c<T, INV>(p.n, X, g.H, nouter, tab.tw[1], mask, st)) return BRI17_OK;
    const int TB = (int)std::min<int64_t>(kP2Threads / p.T, nouter * g.H);
    const int pitch = exchange_pitch(p.n, TB, (int)sizeof(cplx<T>), true);
    const size_t smem = (p.n + (size_t)TB * pitch) * sizeof(cplx<T>);
    const int64_t nl = nouter * g.H;
    launch_pdl(axis_c2c_p2<T, INV, RtEng>, (unsigned)((nl + TB - 1) / TB), p.T * TB, smem, st, X,
               g.H, nl, TB, RtEng{p}, tab.tw[1], pitch, mask);
    return BRI17_OK;
  }
  const int n = g.n[1];
  const int64_t B = g.H;
  const int pitch = n + 1;
  int TB = (int)std::min<int64_t>(B, std::max(4, std::min(32, kTileElems / n)));
  size_t smem = n * sizeof(cplx<T>) + 2 * (size_t)TB * pitch * sizeof(cplx<T>);
  dim3 grid((unsigned)((B + TB - 1) / TB), (unsigned)nouter);
  launch_pdl(axis_c2c<T, INV>, grid, kThreads, smem, st, X, n, B, TB, pitch, g.plan[1], tab.tw[1],
                                                mask);
  return BRI17_OK;
}

// BRI17_FUSED_FORM=registers|staged|tma|tma_registers overrides the
// per-handle choice of the axis-0 form (for measurements); -1 when unset.
static int env_fused_form() {
  static const int form = [] {
    const char* e = getenv("BRI17_FUSED_FORM");
    if (!e) return -1;
    return strcmp(e, "registers") == 0       ? 0
           : strcmp(e, "staged") == 0        ? 1
           : strcmp(e, "tma") == 0           ? 2
           : strcmp(e, "tma_registers") == 0 ? 3
                                             : -1;
  }();
  return form;
}

template <typename T, int DIM, int MODE>
static int launch_fused(const Geometry& g, cplx<T>* X, int batch,
                        int64_t bstride, const FusedParams<T>& fp, BatchMask mask,
                        cudaStream_t st) {
  constexpr int SYM = DIM == 2 ? 3 : 6;
  constexpr int CIN = (MODE == kModeRhs || MODE == kModeSolve) ? SYM : DIM;
  constexpr int COUT = (MODE == kModeStrain || MODE == kModeSolve) ? SYM : DIM;
  constexpr int CMAX = CIN > COUT ? CIN : COUT;
  if (MODE == kModeStiffness && g.use_p8[0]) {
    const Plan8& p = g.p8[0];
    // Form chosen per handle (fused_form, autotuned at creation for FP32);
    // BRI17_FUSED_FORM=registers|staged|tma|tma_registers overrides it (for measurements).
    // A form whose launcher declines the size falls through to the next.
    const int env_form = env_fused_form();
    const int form = env_form >= 0 ? env_form : fp.form;
    if constexpr (std::is_same<T, float>::value && DIM == 3) {
      if ((form == 2 || form == 3) &&
          ct_axis0_stiffness_tma_f32(p.n, form == 3 && !fp.cg, X, g.P, g.cspec, bstride, batch,
                                     fp, mask, st))
        return BRI17_OK;
    }
    if constexpr (std::is_same<T, float>::value) {
      // cg_pq_fusable admits only layouts the TMA-staged form takes.
      if (fp.cg) {
        set_error("internal: p.Kp in the stiffness pass needs the TMA-staged form");
        return BRI17_ERR_UNSUPPORTED_SIZE;
      }
    }
    if (form == 1 &&
        ct_axis0_stiffness_staged<T, DIM>(p.n, X, g.P, g.cspec, bstride, batch, fp, mask, st))
      return BRI17_OK;
    if (ct_axis0_stiffness<T, DIM>(p.n, X, g.P, g.cspec, bstride, batch, fp, mask, st))
      return BRI17_OK;
    const int TB = (int)std::max<int64_t>(1, std::min<int64_t>(kP2FusedThreads / p.T, g.P));
    const int pitch = exchange_pitch(p.n, TB, (int)sizeof(cplx<T>), true);
    const size_t smem = (p.n + (size_t)TB * pitch) * sizeof(cplx<T>);
    dim3 grid((unsigned)((g.P + TB - 1) / TB), (unsigned)batch);
    launch_pdl(axis0_stiffness_p2<T, DIM, RtEng>, grid, p.T * TB, smem, st,
               X, g.P, g.cspec, bstride, TB, pitch, RtEng{p}, fp, mask);
    return BRI17_OK;
  }
  if (MODE == kModeStiffness && g.use_ct3[0] &&
      ct3_axis0_stiffness<T, DIM>(g.n[0], X, g.P, g.cspec, bstride, batch, fp, mask, st))
    return BRI17_OK;
  const int n0 = g.n[0];
  const int pitch = n0 + 1;
  const size_t per_line = (size_t)(CMAX + 1) * pitch * sizeof(cplx<T>);
  size_t budget = kFusedSmemBudget;
  int TB = (int)std::min<size_t>(16, budget / per_line);
  if (TB < 4) {
    budget = kMaxSmem - n0 * sizeof(cplx<T>) - 1024;
    TB = (int)std::min<size_t>(4, budget / per_line);
  }
  if (TB < 1) {
    set_error("axis-0 tile does not fit in shared memory");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  TB = (int)std::min<int64_t>(TB, g.P);
  size_t smem = n0 * sizeof(cplx<T>) + (size_t)TB * per_line;
  dim3 grid((unsigned)((g.P + TB - 1) / TB), (unsigned)batch);
  launch_pdl(axis0_fused<T, DIM, MODE>, grid, kThreads, smem, st, 
      X, n0, g.P, g.cspec, bstride, TB, pitch, g.plan[0], fp, mask);
  return BRI17_OK;
}

template <typename T>
static FusedParams<T> fused_params(const bri17_op* op, const Tables<T>& tab,
                                   int mode) {
  FusedParams<T> fp;
  fp.tab = tab;
  fp.n1 = op->g.dim == 3 ? op->g.n[1] : 1;
  fp.H = op->g.H;
  const double scaling = op->mu / (1. - 2. * op->nu);
  // The solve mode inverts the reference's unscaled K(k) and normalises the
  // inverse transform by 1/|N|, as the strain mode does.
  const double kscale = mode == kModeSolve ? 1.0 : op->corr;
  fp.s = (T)(scaling * kscale);
  fp.mu = (T)(op->mu * kscale);
  fp.corr = (mode == kModeStrain || mode == kModeSolve) ? (T)(1.0 / (double)op->g.size)
                                                        : (T)op->corr;
  fp.mat = nullptr;
  fp.form = op->fused_form;
  fp.status = op->status_dev;
  if constexpr (std::is_same<T, float>::value) {
    if (mode == kModeStiffness) {
      fp.cg = op->cg_st;
      fp.cg_part = op->cg_part;
    }
  }
  return fp;
}

// ---------------------------------------------------------------------------
// Per-pass timing.

constexpr int kNumPasses = 5;

struct PassTiming {
  struct Rec {
    int pass;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> recs;
  double ms[kNumPasses] = {0, 0, 0, 0, 0};
  int64_t n[kNumPasses] = {0, 0, 0, 0, 0};
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void harvest() {
    for (auto& r : recs) {
      float t = 0.f;
      cudaEventSynchronize(r.b);
      if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
        ms[r.pass] += t;
        n[r.pass] += 1;
      }
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }
  ~PassTiming() {
    harvest();
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Brackets one launch with events when timing is enabled.
struct PassScope {
  PassTiming* t;
  PassTiming::Rec rec;
  cudaStream_t st;
  PassScope(bri17_op* op, int pass, cudaStream_t s)
      : t(reinterpret_cast<PassTiming*>(op->timing)), st(s) {
    if (!t) return;
    rec.pass = pass;
    rec.a = t->get();
    rec.b = t->get();
    cudaEventRecord(rec.a, st);
  }
  ~PassScope() {
    if (!t) return;
    cudaEventRecord(rec.b, st);
    t->recs.push_back(rec);
  }
};

// Generic three- or five-pass pipeline: forward rows (+ axis 1), fused axis
// 0, inverse axis 1 (+ rows).  `in` has cin components per batch entry,
// `out` cout; entry z of the spectrum starts at spec + z * cmax * cspec.
// `flags` (optional) masks batch entries: entry z is skipped when
// flags[z * flag_stride] == 0.
template <typename T, int MODE>
static int run_pipeline(bri17_op* op, const Tables<T>& tab, const T* in,
                        T* out, int batch, void* spec, const T* mat,
                        cudaStream_t st, const int* flags = nullptr,
                        int flag_stride = 0) {
  const Geometry& g = op->g;
  const int dim = g.dim;
  const int sym = dim == 2 ? 3 : 6;
  const int cin = (MODE == kModeRhs || MODE == kModeSolve) ? sym : dim;
  const int cout = (MODE == kModeStrain || MODE == kModeSolve) ? sym : dim;
  const int cmax = cin > cout ? cin : cout;
  const int nlast = g.n[dim - 1];
  const int64_t rows_per_comp = g.size / nlast;
  cplx<T>* S = reinterpret_cast<cplx<T>*>(spec);
  const int64_t bstride = (int64_t)cmax * g.cspec;
  set_smem_attrs<T>();
  // Launch over entries [z0, z0 + nz): one launch when their data are
  // contiguous (c == cmax or a single entry), else one per entry.
  auto mask_at = [&](int z0, int64_t unit) {
    BatchMask m;
    m.flags = flags ? flags + (int64_t)z0 * flag_stride : nullptr;
    m.stride = flag_stride;
    m.unit = unit;
    return m;
  };
  const bool fwd_contig = (cin == cmax) || batch == 1;
  const bool inv_contig = (cout == cmax) || batch == 1;
  for (int z0 = 0; z0 < batch; z0 += fwd_contig ? batch : 1) {
    const int nz = fwd_contig ? batch : 1;
    const T* src = in + (int64_t)z0 * cin * g.size;
    cplx<T>* Sz = S + z0 * bstride;
    {
      PassScope ps(op, 0, st);
      launch_rows_r2c<T>(g, src, Sz, (int64_t)nz * cin * rows_per_comp, tab,
                         mask_at(z0, (int64_t)cin * rows_per_comp), st);
    }
    if (dim == 3) {
      PassScope ps(op, 1, st);
      launch_axis1<T, false>(g, Sz, (int64_t)nz * cin * g.n[0], tab,
                             mask_at(z0, (int64_t)cin * g.n[0]), st);
    }
  }
  FusedParams<T> fp = fused_params<T>(op, tab, MODE);
  fp.mat = mat;
  int rc;
  {
    PassScope ps(op, 2, st);
    if (dim == 3)
      rc = launch_fused<T, 3, MODE>(g, S, batch, bstride, fp, mask_at(0, 1), st);
    else
      rc = launch_fused<T, 2, MODE>(g, S, batch, bstride, fp, mask_at(0, 1), st);
  }
  if (rc != BRI17_OK) return rc;
  for (int z0 = 0; z0 < batch; z0 += inv_contig ? batch : 1) {
    const int nz = inv_contig ? batch : 1;
    T* dst = out + (int64_t)z0 * cout * g.size;
    cplx<T>* Sz = S + z0 * bstride;
    if (dim == 3) {
      PassScope ps(op, 3, st);
      launch_axis1<T, true>(g, Sz, (int64_t)nz * cout * g.n[0], tab,
                            mask_at(z0, (int64_t)cout * g.n[0]), st);
    }
    {
      PassScope ps(op, 4, st);
      launch_rows_c2r<T>(g, Sz, dst, (int64_t)nz * cout * rows_per_comp, tab,
                         mask_at(z0, (int64_t)cout * rows_per_comp), st);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "operator launch");
  return BRI17_OK;
}

int ensure_spectrum(bri17_op* op, int comps) {
  if (op->spec && op->spec_comps >= comps) return BRI17_OK;
  const size_t csz = 2 * scalar_bytes(op);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, (size_t)comps * op->g.cspec * csz);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(spectrum)");
  if (op->spec) {
    cudaDeviceSynchronize();
    cudaFree(op->spec);
  }
  op->spec = p;
  op->spec_comps = comps;
  return BRI17_OK;
}

int apply_stiffness_async(bri17_op* op, const void* u, void* f,
                          cudaStream_t st) {
  int rc = ensure_spectrum(op, op->g.dim);
  if (rc != BRI17_OK) return rc;
  // Float pairs on (bri17_op_set_float_pair): the CG solvers' FP64
  // operator applications (the plain solver's, and the residuals of the
  // reliable updates) run in float pairs too.
  if (op->float_pair)
    return ::run_stiffness_df(op, (const double*)u, (double*)f, op->fused_form_df, st);
  if (op->precision == BRI17_F64)
    return run_pipeline<double, kModeStiffness>(
        op, op->tab64, (const double*)u, (double*)f, 1, op->spec, nullptr, st);
  return run_pipeline<float, kModeStiffness>(
      op, op->tab32, (const float*)u, (float*)f, 1, op->spec, nullptr, st);
}

bool cg_pq_fusable(const bri17_op* op) {
  const Geometry& g = op->g;
  if (op->precision != BRI17_F32 || g.dim != 3 || !g.use_p8[0] || !g.use_p8_row) return false;
  const int env_form = env_fused_form();
  if ((env_form >= 0 ? env_form : op->fused_form) != 2) return false;
  if (g.n[0] < 16 || g.n[0] > 1024) return false;
  return tma_layout_ok<float>(op->spec, g.P, g.cspec, 3 * g.cspec, g.n[0]);
}

int apply_stiffness_cg_async(bri17_op* op, const float* p, float* q, CgState* st, double* part,
                             cudaStream_t s) {
  int rc = ensure_spectrum(op, op->g.dim);
  if (rc != BRI17_OK) return rc;
  op->cg_st = st;
  op->cg_part = part;
  rc = run_pipeline<float, kModeStiffness>(op, op->tab32, p, q, 1, op->spec, nullptr, s);
  op->cg_st = nullptr;
  op->cg_part = nullptr;
  return rc;
}

int apply_stiffness_batched_async(bri17_op* op, int batch, const void* u,
                                  void* f, void* spec, const void* mat,
                                  cudaStream_t st, const int* flags,
                                  int flag_stride) {
  if (op->precision == BRI17_F64)
    return run_pipeline<double, kModeStiffness>(op, op->tab64, (const double*)u,
                                                (double*)f, batch, spec,
                                                (const double*)mat, st, flags,
                                                flag_stride);
  return run_pipeline<float, kModeStiffness>(op, op->tab32, (const float*)u,
                                             (float*)f, batch, spec,
                                             (const float*)mat, st, flags,
                                             flag_stride);
}

int eigenstress_rhs_batched_async(bri17_op* op, int batch, const void* tau,
                                  void* b, void* spec, cudaStream_t st) {
  if (op->precision == BRI17_F64)
    return run_pipeline<double, kModeRhs>(op, op->tab64, (const double*)tau,
                                          (double*)b, batch, spec, nullptr, st);
  return run_pipeline<float, kModeRhs>(op, op->tab32, (const float*)tau,
                                       (float*)b, batch, spec, nullptr, st);
}

// Times the forms of the FP32 axis-0 stiffness pass (registers, staged,
// TMA-staged with staged or register compute) on the handle's own spectrum buffer (its contents are
// irrelevant to the timing) and keeps the fastest.
void autotune_fused_form(bri17_op* op) {
  const Geometry& g = op->g;
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int best_form = 0;
  for (int form = 0; form < 4; form++) {
    op->fused_form = form;
    FusedParams<float> fp = fused_params<float>(op, op->tab32, kModeStiffness);
    BatchMask none;
    none.flags = nullptr;
    none.stride = 0;
    none.unit = 1;
    cplx<float>* S = reinterpret_cast<cplx<float>*>(op->spec);
    float ms = 0.f;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, st);
      if (g.dim == 3)
        launch_fused<float, 3, kModeStiffness>(g, S, 1, (int64_t)g.dim * g.cspec, fp, none, st);
      else
        launch_fused<float, 2, kModeStiffness>(g, S, 1, (int64_t)g.dim * g.cspec, fp, none, st);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) ms += t;  // the first run warms up
    }
    if (ms < best) {
      best = ms;
      best_form = form;
    }
  }
  op->fused_form = best_form;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-mode batch kernels (FP64).  Operation order and rounding follow the
// reference line by line; __dmul_rn / __dadd_rn keep the compiler from
// contracting products into fused multiply-adds the reference does not do.

struct ModalArgs {
  Tables<double> tab;
  int dim;
  int n[3];
  double scaling;  // mu / (1 - 2 nu), include/bri17/bri17.hpp:266
  double mu;
};

__device__ __forceinline__ int wrap(int k, int n) {
  int r = k % n;
  return r < 0 ? r + n : r;
}

// Hooke::modal_stiffness, include/bri17/bri17.hpp:247-292 (real parts).
__device__ void modal_stiffness_dev(const ModalArgs& a, const int* kk,
                                    double* K) {
  double phi[3], chi[3], psi[3];
  for (int i = 0; i < a.dim; i++) {
    phi[i] = a.tab.kphi[i][kk[i]];
    chi[i] = a.tab.kchi[i][kk[i]];
    psi[i] = a.tab.kpsi[i][kk[i]];
  }
  const double s = a.scaling;
  if (a.dim == 2) {
    const double H00 = __dmul_rn(phi[0], chi[1]);
    const double H11 = __dmul_rn(chi[0], phi[1]);
    const double Kd = __dmul_rn(a.mu, __dadd_rn(H00, H11));
    K[0] = __dadd_rn(__dmul_rn(s, H00), Kd);
    K[1] = __dmul_rn(__dmul_rn(s, psi[0]), psi[1]);
    K[2] = K[1];
    K[3] = __dadd_rn(__dmul_rn(s, H11), Kd);
  } else {
    const double H00 = __dmul_rn(__dmul_rn(phi[0], chi[1]), chi[2]);
    const double H11 = __dmul_rn(__dmul_rn(chi[0], phi[1]), chi[2]);
    const double H22 = __dmul_rn(__dmul_rn(chi[0], chi[1]), phi[2]);
    const double Kd = __dmul_rn(a.mu, __dadd_rn(__dadd_rn(H00, H11), H22));
    K[0] = __dadd_rn(__dmul_rn(s, H00), Kd);
    K[1] = __dmul_rn(__dmul_rn(__dmul_rn(s, psi[0]), psi[1]), chi[2]);
    K[2] = __dmul_rn(__dmul_rn(__dmul_rn(s, psi[0]), chi[1]), psi[2]);
    K[3] = K[1];
    K[4] = __dadd_rn(__dmul_rn(s, H11), Kd);
    K[5] = __dmul_rn(__dmul_rn(__dmul_rn(s, chi[0]), psi[1]), psi[2]);
    K[6] = K[2];
    K[7] = K[5];
    K[8] = __dadd_rn(__dmul_rn(s, H22), Kd);
  }
}

// Hooke::modal_strain_displacement, include/bri17/bri17.hpp:212-236.
__device__ void modal_strain_displacement_dev(const ModalArgs& a,
                                              const int* kk, double2* B) {
  double c[3], s[3];
  double sum_alpha = 0.0;
  for (int i = 0; i < a.dim; i++) {
    const double alpha = __ddiv_rn(__dmul_rn(kPi, (double)kk[i]), (double)a.n[i]);
    sum_alpha = __dadd_rn(sum_alpha, alpha);
    c[i] = a.tab.bc[i][kk[i]];
    s[i] = a.tab.bs[i][kk[i]];
  }
  double sn, cs;
  sincos(sum_alpha, &sn, &cs);
  const double pr = -2 * sn, pi = 2 * cs;
  if (a.dim == 2) {
    B[0] = make_double2(__dmul_rn(__dmul_rn(pr, s[0]), c[1]),
                        __dmul_rn(__dmul_rn(pi, s[0]), c[1]));
    B[1] = make_double2(__dmul_rn(__dmul_rn(pr, c[0]), s[1]),
                        __dmul_rn(__dmul_rn(pi, c[0]), s[1]));
  } else {
    B[0] = make_double2(__dmul_rn(__dmul_rn(__dmul_rn(pr, s[0]), c[1]), c[2]),
                        __dmul_rn(__dmul_rn(__dmul_rn(pi, s[0]), c[1]), c[2]));
    B[1] = make_double2(__dmul_rn(__dmul_rn(__dmul_rn(pr, c[0]), s[1]), c[2]),
                        __dmul_rn(__dmul_rn(__dmul_rn(pi, c[0]), s[1]), c[2]));
    B[2] = make_double2(__dmul_rn(__dmul_rn(__dmul_rn(pr, c[0]), c[1]), s[2]),
                        __dmul_rn(__dmul_rn(__dmul_rn(pi, c[0]), c[1]), s[2]));
  }
}

__global__ void modal_stiffness_kernel(ModalArgs a, const int* __restrict__ k,
                                       int64_t n, double2* __restrict__ K) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  int kk[3];
  for (int i = 0; i < a.dim; i++) kk[i] = wrap(k[m * a.dim + i], a.n[i]);
  double Kr[9];
  modal_stiffness_dev(a, kk, Kr);
  const int d2 = a.dim * a.dim;
  for (int i = 0; i < d2; i++) K[m * d2 + i] = make_double2(Kr[i], 0.0);
}

__global__ void modal_strain_kernel(ModalArgs a, const int* __restrict__ k,
                                    int64_t n, double2* __restrict__ B) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  int kk[3];
  for (int i = 0; i < a.dim; i++) kk[i] = wrap(k[m * a.dim + i], a.n[i]);
  double2 b[3];
  modal_strain_displacement_dev(a, kk, b);
  for (int i = 0; i < a.dim; i++) B[m * a.dim + i] = b[i];
}

// Hooke::modal_eigenstress_to_opposite_strain, include/bri17/bri17.hpp:
// 308-355: solve K u = tau . conj(B) (K real SPD for k != 0, factored by a
// real Cholesky), return sym(B (x) u) in Mandel form; k = 0 gives 0.
__global__ void modal_eigenstress_kernel(ModalArgs a, const int* __restrict__ k,
                                         int64_t n,
                                         const double2* __restrict__ tau,
                                         double2* __restrict__ eta) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const int dim = a.dim;
  const int sym = dim == 2 ? 3 : 6;
  int kk[3];
  bool null_frequency = true;
  for (int i = 0; i < dim; i++) {
    const int ki = k[m * dim + i];
    kk[i] = wrap(ki, a.n[i]);
    null_frequency = null_frequency && (ki == 0);
  }
  if (null_frequency) {
    for (int q = 0; q < sym; q++) eta[m * sym + q] = make_double2(0.0, 0.0);
    return;
  }
  double2 B[3];
  double K[9];
  modal_strain_displacement_dev(a, kk, B);
  modal_stiffness_dev(a, kk, K);
  const double ir2 = 0.7071067811865475244008443621048490392848;
  const double r2 = 1.414213562373095048801688724209698079;
  double2 t[3][3];
  const double2* tm = tau + m * sym;
  if (dim == 2) {
    t[0][0] = tm[0];
    t[1][1] = tm[1];
    t[0][1] = t[1][0] = make_double2(tm[2].x * ir2, tm[2].y * ir2);
  } else {
    t[0][0] = tm[0];
    t[1][1] = tm[1];
    t[2][2] = tm[2];
    t[1][2] = t[2][1] = make_double2(tm[3].x * ir2, tm[3].y * ir2);
    t[0][2] = t[2][0] = make_double2(tm[4].x * ir2, tm[4].y * ir2);
    t[0][1] = t[1][0] = make_double2(tm[5].x * ir2, tm[5].y * ir2);
  }
  double2 rhs[3];
  for (int i = 0; i < dim; i++) {
    double sr = 0.0, si = 0.0;
    for (int j = 0; j < dim; j++) {
      const double br = B[j].x, bi = -B[j].y;
      sr += t[i][j].x * br - t[i][j].y * bi;
      si += t[i][j].x * bi + t[i][j].y * br;
    }
    rhs[i] = make_double2(sr, si);
  }
  double Lc[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int j = 0; j < dim; j++) {
    double d = K[j * dim + j];
    for (int p = 0; p < j; p++) d -= Lc[j][p] * Lc[j][p];
    d = sqrt(d);
    Lc[j][j] = d;
    for (int i = j + 1; i < dim; i++) {
      double s = K[i * dim + j];
      for (int p = 0; p < j; p++) s -= Lc[i][p] * Lc[j][p];
      Lc[i][j] = s / d;
    }
  }
  double2 y[3], u[3];
  for (int i = 0; i < dim; i++) {
    double sr = rhs[i].x, si = rhs[i].y;
    for (int p = 0; p < i; p++) {
      sr -= Lc[i][p] * y[p].x;
      si -= Lc[i][p] * y[p].y;
    }
    y[i] = make_double2(sr / Lc[i][i], si / Lc[i][i]);
  }
  for (int i = dim - 1; i >= 0; i--) {
    double sr = y[i].x, si = y[i].y;
    for (int p = i + 1; p < dim; p++) {
      sr -= Lc[p][i] * u[p].x;
      si -= Lc[p][i] * u[p].y;
    }
    u[i] = make_double2(sr / Lc[i][i], si / Lc[i][i]);
  }
  static const int I3[6] = {0, 1, 2, 1, 2, 0}, J3[6] = {0, 1, 2, 2, 0, 1};
  static const int I2[3] = {0, 1, 0}, J2[3] = {0, 1, 1};
  for (int q = 0; q < sym; q++) {
    const int i = dim == 2 ? I2[q] : I3[q];
    const int j = dim == 2 ? J2[q] : J3[q];
    double er = 0.5 * ((B[i].x * u[j].x - B[i].y * u[j].y) +
                       (u[i].x * B[j].x - u[i].y * B[j].y));
    double ei = 0.5 * ((B[i].x * u[j].y + B[i].y * u[j].x) +
                       (u[i].x * B[j].y + u[i].y * B[j].x));
    if (i != j) {
      er *= r2;
      ei *= r2;
    }
    eta[m * sym + q] = make_double2(er, ei);
  }
}

static ModalArgs modal_args(const bri17_op* op) {
  ModalArgs a;
  a.tab = op->tab64;
  a.dim = op->g.dim;
  for (int i = 0; i < 3; i++) a.n[i] = op->g.n[i];
  a.scaling = op->mu / (1. - 2. * op->nu);
  a.mu = op->mu;
  return a;
}

static int check_material(double mu, double nu) {
  if (!(mu > 0) || !isfinite(mu)) return invalid("mu must be positive and finite");
  if (!(nu > -1.0 && nu < 0.5)) return invalid("nu must lie in (-1, 0.5)");
  return BRI17_OK;
}

}  // namespace bri17gb

using namespace bri17gb;

// ---------------------------------------------------------------------------
// C ABI.

extern "C" const char* bri17_status_string(int s) {
  switch (s) {
    case BRI17_OK: return "ok";
    case BRI17_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BRI17_ERR_UNSUPPORTED_SIZE: return "unsupported size";
    case BRI17_ERR_CUDA: return "CUDA error";
    case BRI17_ERR_OUT_OF_MEMORY: return "out of device memory";
    case BRI17_ERR_NOT_CONVERGED: return "not converged";
    case BRI17_ERR_BREAKDOWN: return "breakdown (NaN/Inf or loss of positivity)";
    case BRI17_ERR_NO_DEVICE: return "no CUDA device";
    case BRI17_ERR_BUSY: return "busy";
    case BRI17_ERR_NOT_FOUND: return "not found";
    case BRI17_ERR_CANCELLED: return "cancelled";
    case BRI17_ERR_TIMEOUT: return "a bounded device wait ran out (results invalid)";
    case BRI17_ERR_STAGNATED: return "residual stagnated above the tolerance";
    default: return "unknown status";
  }
}

extern "C" const char* bri17_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* bri17_version(void) { return "0.1.0"; }

extern "C" int bri17_op_create(int dim, const int* shape, const double* L,
                               double mu, double nu, int precision,
                               bri17_op** out) {
  if (!out || !shape || !L) return invalid("null pointer");
  *out = nullptr;
  if (dim != 2 && dim != 3) return invalid("dim must be 2 or 3");
  if (precision != BRI17_F64 && precision != BRI17_F32)
    return invalid("precision must be BRI17_F64 or BRI17_F32");
  int rc = check_material(mu, nu);
  if (rc != BRI17_OK) return rc;
  for (int i = 0; i < dim; i++) {
    if (shape[i] < 1) return invalid("shape entries must be >= 1");
    if (!(L[i] > 0) || !isfinite(L[i])) return invalid("L entries must be positive");
    if (shape[i] > 1024) {
      set_error("axis length above 1024");
      return BRI17_ERR_UNSUPPORTED_SIZE;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device visible");
    return BRI17_ERR_NO_DEVICE;
  }
  bri17_op* op = new bri17_op();
  memset(op, 0, sizeof(*op));
  Geometry& g = op->g;
  g.dim = dim;
  g.size = 1;
  for (int i = 0; i < 3; i++) {
    g.n[i] = i < dim ? shape[i] : 1;
    op->L[i] = i < dim ? L[i] : 1.0;
  }
  for (int i = 0; i < dim; i++) g.size *= shape[i];
  if (g.size > ((int64_t)1 << 31) - 1) {
    delete op;
    set_error("grid larger than 2^31 - 1 nodes (CartesianGrid::size is int)");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  const int nl = g.n[dim - 1];
  g.H = nl / 2 + 1;
  g.P = dim == 3 ? (int64_t)g.n[1] * g.H : (int64_t)g.H;
  g.cspec = (int64_t)g.n[0] * g.P;
  bool ok = make_plan(nl % 2 == 0 ? nl / 2 : nl, &g.plan_row);
  for (int i = 0; i < dim; i++) ok = ok && make_plan(g.n[i], &g.plan[i]);
  set_p8_plans(&g);
  if (!ok) {
    delete op;
    set_error("axis length has a prime factor above 61");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  op->mu = mu;
  op->nu = nu;
  op->precision = precision;
  cudaGetDevice(&op->device);
  double cv = 1.0;
  for (int i = 0; i < dim; i++) cv *= op->L[i] / g.n[i];
  op->cell_volume = cv;
  op->corr = cv / (double)g.size;

  std::vector<HostTables> ht(dim);
  for (int i = 0; i < dim; i++) host_tables(g.n[i], op->L[i], &ht[i]);
  const size_t b64 = tables_bytes(g.n, dim, sizeof(double));
  const size_t b32 = precision == BRI17_F32 ? tables_bytes(g.n, dim, sizeof(float)) : 0;
  std::vector<unsigned char> host(b64 + b32 + 16);
  cudaError_t e = cudaMalloc(&op->table_mem, b64 + b32 + 16);
  if (e != cudaSuccess) {
    delete op;
    return cuda_fail(e, "cudaMalloc(tables)");
  }
  size_t off = 0;
  unsigned char* dev = (unsigned char*)op->table_mem;
  fill_tables<double>(ht, g.n, dim, host.data(), &off, &op->tab64, dev);
  if (precision == BRI17_F32)
    fill_tables<float>(ht, g.n, dim, host.data(), &off, &op->tab32, dev);
  e = cudaMemcpy(op->table_mem, host.data(), off, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(op->table_mem);
    delete op;
    return cuda_fail(e, "cudaMemcpy(tables)");
  }
  e = cudaHostAlloc((void**)&op->status_host, 4 * sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess)
    e = cudaHostGetDevicePointer((void**)&op->status_dev, op->status_host, 0);
  if (e != cudaSuccess) {
    cudaFreeHost(op->status_host);
    cudaFree(op->table_mem);
    delete op;
    return cuda_fail(e, "cudaHostAlloc(status words)");
  }
  memset(op->status_host, 0, 4 * sizeof(int));
  rc = ensure_spectrum(op, dim);
  if (rc != BRI17_OK) {
    cudaFreeHost(op->status_host);
    cudaFree(op->table_mem);
    delete op;
    return rc;
  }
  // Kernel attributes are set before any stream capture can begin.
  if (precision == BRI17_F64)
    set_smem_attrs<double>();
  else
    set_smem_attrs<float>();
  if (precision == BRI17_F32 && g.use_p8[0]) autotune_fused_form(op);
  op->mode_mu = new std::mutex();
  *out = op;
  return BRI17_OK;
}

extern "C" int bri17_op_destroy(bri17_op* op) {
  if (!op) return BRI17_OK;
  cudaDeviceSynchronize();
  if (op->twin32) bri17_op_destroy(op->twin32);
  cudaFree(op->table_mem);
  cudaFree(op->table_df);
  cudaFree(op->spec);
  cudaFree(op->stage_in);
  cudaFree(op->stage_out);
  if (op->copy_stream) {
    cudaStreamDestroy(op->copy_stream);
    for (int i = 0; i < kHostEvents; i++) cudaEventDestroy(op->host_events[i]);
  }
  if (op->cg_work && op->cg_free) op->cg_free(op->cg_work);
  delete reinterpret_cast<PassTiming*>(op->timing);
  cudaFreeHost(op->status_host);
  cudaFreeHost(op->mode_stage_host);
  if (op->mode_stream) cudaStreamDestroy(op->mode_stream);
  delete op->mode_mu;
  delete op;
  return BRI17_OK;
}

extern "C" int bri17_op_info(const bri17_op* op, int64_t* size,
                             int64_t* workspace_bytes) {
  if (!op) return invalid("null handle");
  if (size) *size = op->g.size;
  if (workspace_bytes)
    *workspace_bytes = (int64_t)op->spec_comps * op->g.cspec * 2 * scalar_bytes(op);
  return BRI17_OK;
}

extern "C" int bri17_op_set_material(bri17_op* op, double mu, double nu) {
  if (!op) return invalid("null handle");
  int rc = check_material(mu, nu);
  if (rc != BRI17_OK) return rc;
  op->mu = mu;
  op->nu = nu;
  op->material_epoch++;
  if (op->twin32) bri17_op_set_material(op->twin32, mu, nu);
  return BRI17_OK;
}

extern "C" int bri17_modal_stiffness_batch(const bri17_op* op, const int* k,
                                           int64_t n, void* K, void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  if (n < 0) return invalid("negative count");
  if (n == 0) return BRI17_OK;
  if (!k || !K) return invalid("null pointer");
  ModalArgs a = modal_args(op);
  modal_stiffness_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      a, k, n, (double2*)K);
  BRI17_CUDA_TRY(cudaGetLastError());
  return BRI17_OK;
}

extern "C" int bri17_modal_strain_displacement_batch(const bri17_op* op,
                                                     const int* k, int64_t n,
                                                     void* B, void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  if (n < 0) return invalid("negative count");
  if (n == 0) return BRI17_OK;
  if (!k || !B) return invalid("null pointer");
  ModalArgs a = modal_args(op);
  modal_strain_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      a, k, n, (double2*)B);
  BRI17_CUDA_TRY(cudaGetLastError());
  return BRI17_OK;
}

extern "C" int bri17_modal_eigenstress_to_opposite_strain_batch(
    const bri17_op* op, const int* k, int64_t n, const void* tau, void* eta,
    void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  if (n < 0) return invalid("negative count");
  if (n == 0) return BRI17_OK;
  if (!k || !tau || !eta) return invalid("null pointer");
  ModalArgs a = modal_args(op);
  modal_eigenstress_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      a, k, n, (const double2*)tau, (double2*)eta);
  BRI17_CUDA_TRY(cudaGetLastError());
  return BRI17_OK;
}

// ---------------------------------------------------------------------------
// Per-mode functions on host buffers.

namespace bri17gb {

// Runs launch(k_dev, in_dev, out_dev, stream) on the handle's private stream
// over page-locked staging mapped into the device: k (n x dim int32) and
// `in` are copied into the staging, the kernel reads and writes it in
// place (over the host link), and `out` is copied back once the stream has
// synchronised.  No device allocation after the first call of a given size.
template <typename Launch>
static int modal_host_call(const bri17_op* cop, const int* k, int64_t n, const void* in,
                           size_t in_bytes, void* out, size_t out_bytes, Launch&& launch) {
  bri17_op* op = const_cast<bri17_op*>(cop);
  std::lock_guard<std::mutex> lock(*op->mode_mu);
  const size_t k_bytes = align16((size_t)n * op->g.dim * sizeof(int));
  const size_t need = k_bytes + align16(in_bytes) + out_bytes;
  if (op->mode_stage_bytes < need) {
    cudaFreeHost(op->mode_stage_host);
    op->mode_stage_host = op->mode_stage_dev = nullptr;
    op->mode_stage_bytes = 0;
    const size_t bytes = std::max<size_t>(need, 4096);
    BRI17_CUDA_TRY(cudaHostAlloc((void**)&op->mode_stage_host, bytes, cudaHostAllocMapped));
    BRI17_CUDA_TRY(cudaHostGetDevicePointer((void**)&op->mode_stage_dev, op->mode_stage_host, 0));
    op->mode_stage_bytes = bytes;
  }
  if (!op->mode_stream)
    BRI17_CUDA_TRY(cudaStreamCreateWithFlags(&op->mode_stream, cudaStreamNonBlocking));
  memcpy(op->mode_stage_host, k, (size_t)n * op->g.dim * sizeof(int));
  if (in_bytes) memcpy(op->mode_stage_host + k_bytes, in, in_bytes);
  unsigned char* d = op->mode_stage_dev;
  launch((const int*)d, (const void*)(d + k_bytes), (void*)(d + k_bytes + align16(in_bytes)),
         op->mode_stream);
  BRI17_CUDA_TRY(cudaGetLastError());
  BRI17_CUDA_TRY(cudaStreamSynchronize(op->mode_stream));
  memcpy(out, op->mode_stage_host + k_bytes + align16(in_bytes), out_bytes);
  return BRI17_OK;
}

static int modal_host_checks(const bri17_op* op, const int* k, int64_t n, const void* out) {
  if (!op) return invalid("null handle");
  const int dc = check_device(op);
  if (dc != BRI17_OK) return dc;
  if (n < 0) return invalid("negative count");
  if (n > 0 && (!k || !out)) return invalid("null pointer");
  return BRI17_OK;
}

}  // namespace bri17gb

extern "C" int bri17_modal_stiffness_host(const bri17_op* op, const int* k, int64_t n,
                                          void* K) {
  int rc = modal_host_checks(op, k, n, K);
  if (rc != BRI17_OK || n == 0) return rc;
  const ModalArgs a = modal_args(op);
  const int d2 = op->g.dim * op->g.dim;
  return modal_host_call(op, k, n, nullptr, 0, K, (size_t)n * d2 * sizeof(double2),
                         [&](const int* kd, const void*, void* o, cudaStream_t st) {
                           modal_stiffness_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                               a, kd, n, (double2*)o);
                         });
}

extern "C" int bri17_modal_strain_displacement_host(const bri17_op* op, const int* k,
                                                    int64_t n, void* B) {
  int rc = modal_host_checks(op, k, n, B);
  if (rc != BRI17_OK || n == 0) return rc;
  const ModalArgs a = modal_args(op);
  return modal_host_call(op, k, n, nullptr, 0, B, (size_t)n * op->g.dim * sizeof(double2),
                         [&](const int* kd, const void*, void* o, cudaStream_t st) {
                           modal_strain_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                               a, kd, n, (double2*)o);
                         });
}

extern "C" int bri17_modal_eigenstress_to_opposite_strain_host(const bri17_op* op,
                                                               const int* k, int64_t n,
                                                               const void* tau, void* eta) {
  int rc = modal_host_checks(op, k, n, eta);
  if (rc != BRI17_OK || n == 0) return rc;
  if (!tau) return invalid("null pointer");
  const ModalArgs a = modal_args(op);
  const int sym = op->g.dim == 2 ? 3 : 6;
  const size_t bytes = (size_t)n * sym * sizeof(double2);
  return modal_host_call(op, k, n, tau, bytes, eta, bytes,
                         [&](const int* kd, const void* t, void* o, cudaStream_t st) {
                           modal_eigenstress_kernel<<<(unsigned)((n + 127) / 128), 128, 0,
                                                      st>>>(a, kd, n, (const double2*)t,
                                                            (double2*)o);
                         });
}

// ---------------------------------------------------------------------------
// Float-pair (df64) stiffness operator on FP64 handles.

// The five passes in float-pair arithmetic (3D, compile-time lengths
// only).  `form` selects the axis-0 pass: 2 TMA-staged, else staged.
// `mat` (optional, device): the (s, mu) pair of this application as float
// pairs, overriding the handle's material (the server's slots).
static int run_stiffness_df(bri17_op* op, const double* u, double* f, int form,
                            cudaStream_t st, const df64* mat) {
  if (env_fused_form() >= 0) form = env_fused_form();
  const Geometry& g = op->g;
  const int dim = g.dim;
  const Tables<df64>& tab = op->tabdf;
  cplx<df64>* S = reinterpret_cast<cplx<df64>*>(op->spec);
  BatchMask none;
  none.flags = nullptr;
  none.stride = 0;
  none.unit = 1;
  const int nl = g.n[dim - 1];
  const int64_t rows = (int64_t)dim * (g.size / nl);
  bool ok;
  {
    PassScope ps(op, 0, st);
    ok = ct_rows_r2c<df64>(nl / 2, u, S, rows, g.H, tab.tw[dim - 1], none, st);
  }
  if (ok && dim == 3) {
    PassScope ps(op, 1, st);
    ok = ct_axis_c2c<df64, false>(g.n[1], S, g.H, (int64_t)dim * g.n[0], tab.tw[1], none, st);
  }
  if (ok) {
    PassScope ps(op, 2, st);
    FusedParams<df64> fp = fused_params<df64>(op, tab, kModeStiffness);
    fp.mat = mat;
    const int64_t bstride = (int64_t)dim * g.cspec;
    bool done = false;
    if (form == 2 && dim == 3)
      done = ct_axis0_stiffness_tma_df(g.n[0], S, g.P, g.cspec, bstride, 1, fp, none, st);
    if (!done && dim == 3)
      done = ct_axis0_stiffness_staged<df64, 3>(g.n[0], S, g.P, g.cspec, bstride, 1, fp, none,
                                                st);
    if (!done && dim == 2)
      done = ct_axis0_stiffness_staged<df64, 2>(g.n[0], S, g.P, g.cspec, bstride, 1, fp, none,
                                                st);
    ok = done;
  }
  if (ok && dim == 3) {
    PassScope ps(op, 3, st);
    ok = ct_axis_c2c<df64, true>(g.n[1], S, g.H, (int64_t)dim * g.n[0], tab.tw[1], none, st);
  }
  if (ok) {
    PassScope ps(op, 4, st);
    ok = ct_rows_c2r<df64>(nl / 2, S, f, rows, g.H, tab.tw[dim - 1], none, st);
  }
  if (!ok) {
    set_error("float-pair operator: no compiled instance for this grid");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "float-pair operator launch");
  return BRI17_OK;
}

// Whether every pass of the grid has a compile-time float-pair instance:
// power-of-two axes, the strided ones (shape[0], and shape[1] in 3D) in
// 64..512, the last one in 128..1024.
static bool float_pair_supported(const Geometry& g) {
  for (int i = 0; i < g.dim - 1; i++)
    if (!is_pow2(g.n[i]) || g.n[i] < 64 || g.n[i] > 512) return false;
  const int nl = g.n[g.dim - 1];
  return is_pow2(nl) && nl >= 128 && nl <= 1024;
}

// Times the axis-0 forms of the float-pair operator on the handle's own
// buffers and keeps the fastest (as autotune_fused_form does for FP32).
static void autotune_df_form(bri17_op* op) {
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  void* u = nullptr;
  const size_t bytes = (size_t)op->g.dim * op->g.size * sizeof(double);
  if (cudaMalloc(&u, bytes) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamDestroy(st);
    return;
  }
  cudaMemsetAsync(u, 0, bytes, st);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int best_form = 1;
  for (int form = 1; form <= 2; form++) {
    float ms = 0.f;
    bool ok = true;
    for (int rep = 0; rep < 3 && ok; rep++) {
      cudaEventRecord(e0, st);
      ok = run_stiffness_df(op, (const double*)u, (double*)u, form, st) == BRI17_OK;
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) ms += t;
    }
    if (ok && ms < best) {
      best = ms;
      best_form = form;
    }
  }
  op->fused_form_df = best_form;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(u);
  cudaStreamDestroy(st);
  cudaGetLastError();
}

static int ensure_float_pair_tables(bri17_op* op);

extern "C" int bri17_op_set_float_pair(bri17_op* op, int enable) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  if (!enable) {
    if (op->float_pair) op->material_epoch++;  // captured CG graphs hold the old form
    op->float_pair = false;
    return BRI17_OK;
  }
  if (op->precision != BRI17_F64) return invalid("float-pair arithmetic needs an FP64 handle");
  if (!float_pair_supported(op->g)) {
    set_error("float-pair operator: power-of-two grids, the strided axes in 64..512, the "
              "last axis in 128..1024");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  const int rc = ensure_float_pair_tables(op);
  if (rc != BRI17_OK) return rc;
  if (!op->float_pair) op->material_epoch++;  // captured CG graphs hold the old form
  op->float_pair = true;
  return BRI17_OK;
}

// Float-pair tables, kernel attributes and axis-0 form of an FP64 handle
// whose grid has float-pair instances (built once).
static int ensure_float_pair_tables(bri17_op* op) {
  if (!op->table_df) {
    const Geometry& g = op->g;
    std::vector<HostTables> ht(g.dim);
    for (int i = 0; i < g.dim; i++) host_tables(g.n[i], op->L[i], &ht[i]);
    const size_t b = tables_bytes(g.n, g.dim, sizeof(df64));
    std::vector<unsigned char> host(b + 16);
    void* mem = nullptr;
    cudaError_t e = cudaMalloc(&mem, b + 16);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(float-pair tables)");
    size_t off = 0;
    fill_tables<df64>(ht, g.n, g.dim, host.data(), &off, &op->tabdf, (unsigned char*)mem);
    e = cudaMemcpy(mem, host.data(), off, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(mem);
      return cuda_fail(e, "cudaMemcpy(float-pair tables)");
    }
    op->table_df = mem;
    static std::atomic<unsigned long long> done{0};
    once_per_device(&done, [] {
      ct_set_smem_attrs_df_rows(kMaxSmem);
      ct_set_smem_attrs_df_c2c(kMaxSmem);
      ct_set_smem_attrs_df_axis0(kMaxSmem);
    });
    const int rc = ensure_spectrum(op, op->g.dim);
    if (rc != BRI17_OK) return rc;
    autotune_df_form(op);
  }
  return BRI17_OK;
}

int bri17gb::prepare_accurate_residual(bri17_op* op) {
  static const bool f64_only = [] {
    const char* e = getenv("BRI17_MIXED_RESIDUAL");
    return e && strcmp(e, "f64") == 0;
  }();
  op->residual_df = false;
  if (f64_only || op->float_pair || op->precision != BRI17_F64 ||
      !float_pair_supported(op->g))
    return BRI17_OK;
  const int rc = ensure_float_pair_tables(op);
  if (rc != BRI17_OK) return rc;
  op->residual_df = true;
  return BRI17_OK;
}

int bri17gb::apply_accurate_mat_async(bri17_op* op, const double* u, double* f,
                                      const void* mat_df, cudaStream_t st) {
  if (!op->residual_df) {
    set_error("internal: float-pair residual not prepared");
    return BRI17_ERR_UNSUPPORTED_SIZE;
  }
  const int rc = ensure_spectrum(op, op->g.dim);
  if (rc != BRI17_OK) return rc;
  return ::run_stiffness_df(op, u, f, op->fused_form_df, st, static_cast<const df64*>(mat_df));
}

int bri17gb::apply_accurate_async(bri17_op* op, const double* u, double* f, cudaStream_t st) {
  if (op->residual_df && !op->float_pair) {
    const int rc = ensure_spectrum(op, op->g.dim);
    if (rc != BRI17_OK) return rc;
    return ::run_stiffness_df(op, u, f, op->fused_form_df, st);
  }
  return apply_stiffness_async(op, u, f, st);
}

extern "C" int bri17_apply_stiffness(bri17_op* op, const void* u, void* f,
                                     void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  {
    const int ts = take_status(op);  // a failure of earlier work on the handle
    if (ts != BRI17_OK) return ts;
  }
  if (!u || !f) return invalid("null pointer");
  if (op->float_pair) {
    const int rc = ensure_spectrum(op, op->g.dim);
    if (rc != BRI17_OK) return rc;
    return run_stiffness_df(op, (const double*)u, (double*)f, op->fused_form_df,
                            (cudaStream_t)stream);
  }
  return apply_stiffness_async(op, u, f, (cudaStream_t)stream);
}

// f = K u from host buffers, pipelined in chunks of axis-0 planes (one
// chunk per component: finer chunks leave the GPU under-filled): the
// copy stream uploads chunk j while the compute stream runs the last-axis
// and axis-1 passes of chunk j-1 (both only need whole planes), and
// downloads chunk j while the inverse passes of chunk j+1 run.  Only the
// axis-0 pass needs all of the field at once.
constexpr int kHostChunksPerComp = 1;  // finer chunks measured slower (launch tails)

// Device address of a page-locked host buffer, or nullptr for memory the
// runtime does not know as page-locked (pageable memory takes the copy
// pipeline).
static const void* device_view(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

template <typename T>
static int apply_host_pipelined(bri17_op* op, const T* u_host, T* f_host,
                                cudaStream_t st) {
  const Geometry& g = op->g;
  const int dim = g.dim;
  const int n0 = g.n[0];
  // Elements of one axis-0 plane: real field, spectrum rows, spectrum.
  const int64_t plane_real = g.size / n0;
  const int64_t plane_rows = plane_real / g.n[dim - 1];
  const int64_t plane_spec = g.cspec / n0;
  const int per = std::max(1, (n0 + kHostChunksPerComp - 1) / kHostChunksPerComp);
  const Tables<T>& tab = *reinterpret_cast<const Tables<T>*>(
      op->precision == BRI17_F64 ? (const void*)&op->tab64 : (const void*)&op->tab32);
  T* din = reinterpret_cast<T*>(op->stage_in);
  T* dout = reinterpret_cast<T*>(op->stage_out);
  cplx<T>* S = reinterpret_cast<cplx<T>*>(op->spec);
  cudaEvent_t* ev = op->host_events;
  BatchMask none;
  none.flags = nullptr;
  none.stride = 0;
  none.unit = 1;
  set_smem_attrs<T>();
  cudaStream_t cp = op->copy_stream;
  BRI17_CUDA_TRY(cudaEventRecord(ev[0], st));
  BRI17_CUDA_TRY(cudaStreamWaitEvent(cp, ev[0], 0));
  int nev = 0;
  auto next_event = [&]() { return ev[1 + (nev++ % (kHostEvents - 1))]; };
  // Forward: per chunk, upload then last-axis (+ axis-1) passes.
  for (int c = 0; c < dim; c++) {
    for (int p0 = 0; p0 < n0; p0 += per) {
      const int np = std::min(per, n0 - p0);
      const int64_t roff = c * g.size + p0 * plane_real;
      BRI17_CUDA_TRY(cudaMemcpyAsync(din + roff, u_host + roff, np * plane_real * sizeof(T),
                                     cudaMemcpyHostToDevice, cp));
      cudaEvent_t e = next_event();
      BRI17_CUDA_TRY(cudaEventRecord(e, cp));
      BRI17_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
      cplx<T>* Sc = S + c * g.cspec + p0 * plane_spec;
      {
        PassScope ps(op, 0, st);
        launch_rows_r2c<T>(g, din + roff, Sc, np * plane_rows, tab, none, st);
      }
      if (dim == 3) {
        PassScope ps(op, 1, st);
        launch_axis1<T, false>(g, Sc, np, tab, none, st);
      }
    }
  }
  FusedParams<T> fp = fused_params<T>(op, tab, kModeStiffness);
  int rc;
  {
    PassScope ps(op, 2, st);
    if (dim == 3)
      rc = launch_fused<T, 3, kModeStiffness>(g, S, 1, (int64_t)dim * g.cspec, fp, none, st);
    else
      rc = launch_fused<T, 2, kModeStiffness>(g, S, 1, (int64_t)dim * g.cspec, fp, none, st);
  }
  if (rc != BRI17_OK) return rc;
  // Inverse: per chunk, axis-1 (+ last-axis) passes then download.
  for (int c = 0; c < dim; c++) {
    for (int p0 = 0; p0 < n0; p0 += per) {
      const int np = std::min(per, n0 - p0);
      const int64_t roff = c * g.size + p0 * plane_real;
      cplx<T>* Sc = S + c * g.cspec + p0 * plane_spec;
      if (dim == 3) {
        PassScope ps(op, 3, st);
        launch_axis1<T, true>(g, Sc, np, tab, none, st);
      }
      {
        PassScope ps(op, 4, st);
        launch_rows_c2r<T>(g, Sc, dout + roff, np * plane_rows, tab, none, st);
      }
      cudaEvent_t e = next_event();
      BRI17_CUDA_TRY(cudaEventRecord(e, st));
      BRI17_CUDA_TRY(cudaStreamWaitEvent(cp, e, 0));
      BRI17_CUDA_TRY(cudaMemcpyAsync(f_host + roff, dout + roff, np * plane_real * sizeof(T),
                                     cudaMemcpyDeviceToHost, cp));
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "operator launch");
  BRI17_CUDA_TRY(cudaStreamSynchronize(cp));
  return BRI17_OK;
}

extern "C" int bri17_apply_stiffness_host(bri17_op* op, const void* u_host,
                                          void* f_host, void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  {
    const int ts = take_status(op);  // a failure of earlier work on the handle
    if (ts != BRI17_OK) return ts;
  }
  if (!u_host || !f_host) return invalid("null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = (size_t)op->g.dim * op->g.size * scalar_bytes(op);
  if (op->stage_bytes < bytes) {
    cudaFree(op->stage_in);
    cudaFree(op->stage_out);
    op->stage_in = op->stage_out = nullptr;
    op->stage_bytes = 0;
    BRI17_CUDA_TRY(cudaMalloc(&op->stage_in, bytes));
    BRI17_CUDA_TRY(cudaMalloc(&op->stage_out, bytes));
    op->stage_bytes = bytes;
  }
  if (!op->copy_stream) {
    BRI17_CUDA_TRY(cudaStreamCreateWithFlags(&op->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < kHostEvents; i++)
      BRI17_CUDA_TRY(cudaEventCreateWithFlags(&op->host_events[i], cudaEventDisableTiming));
  }
  int rc = ensure_spectrum(op, op->g.dim);
  if (rc != BRI17_OK) return rc;
  // Page-locked host buffers are addressable from the GPU (over NVLink-C2C
  // on Grace machines): the first pass then reads u and the last pass writes
  // f in host memory directly, and the link traffic overlaps those passes'
  // compute instead of running as separate copies before and after them.
  // BRI17_HOST_PATH=staged forces the copy pipeline (for measurements).
  static const bool force_staged = [] {
    const char* e = getenv("BRI17_HOST_PATH");
    return e && strcmp(e, "staged") == 0;
  }();
  const void* du = force_staged ? nullptr : device_view(u_host);
  void* df = force_staged ? nullptr : const_cast<void*>(device_view(f_host));
  if (du && df) {
    if (op->float_pair)
      rc = run_stiffness_df(op, (const double*)du, (double*)df, op->fused_form_df, st);
    else if (op->precision == BRI17_F64)
      rc = run_pipeline<double, kModeStiffness>(op, op->tab64, (const double*)du, (double*)df,
                                                1, op->spec, nullptr, st);
    else
      rc = run_pipeline<float, kModeStiffness>(op, op->tab32, (const float*)du, (float*)df, 1,
                                               op->spec, nullptr, st);
    if (rc != BRI17_OK) return rc;
    BRI17_CUDA_TRY(cudaStreamSynchronize(st));
    return take_status(op);
  }
  if (op->float_pair) {
    // Pageable buffers: whole-field copies around the float-pair passes.
    const size_t bytes = (size_t)op->g.dim * op->g.size * sizeof(double);
    BRI17_CUDA_TRY(cudaMemcpyAsync(op->stage_in, u_host, bytes, cudaMemcpyHostToDevice, st));
    rc = run_stiffness_df(op, (const double*)op->stage_in, (double*)op->stage_out,
                          op->fused_form_df, st);
    if (rc != BRI17_OK) return rc;
    BRI17_CUDA_TRY(cudaMemcpyAsync(f_host, op->stage_out, bytes, cudaMemcpyDeviceToHost, st));
    BRI17_CUDA_TRY(cudaStreamSynchronize(st));
    return take_status(op);
  }
  if (op->precision == BRI17_F64)
    rc = apply_host_pipelined<double>(op, (const double*)u_host, (double*)f_host, st);
  else
    rc = apply_host_pipelined<float>(op, (const float*)u_host, (float*)f_host, st);
  if (rc != BRI17_OK) return rc;
  return take_status(op);
}

extern "C" int bri17_apply_strain(bri17_op* op, const void* u, void* eps,
                                  void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  {
    const int ts = take_status(op);  // a failure of earlier work on the handle
    if (ts != BRI17_OK) return ts;
  }
  if (!u || !eps) return invalid("null pointer");
  const int sym = op->g.dim == 2 ? 3 : 6;
  int rc = ensure_spectrum(op, sym);
  if (rc != BRI17_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (op->precision == BRI17_F64)
    return run_pipeline<double, kModeStrain>(op, op->tab64, (const double*)u,
                                             (double*)eps, 1, op->spec, nullptr, st);
  return run_pipeline<float, kModeStrain>(op, op->tab32, (const float*)u,
                                          (float*)eps, 1, op->spec, nullptr, st);
}

extern "C" int bri17_eigenstress_rhs(bri17_op* op, const void* tau, void* b,
                                     void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  {
    const int ts = take_status(op);  // a failure of earlier work on the handle
    if (ts != BRI17_OK) return ts;
  }
  if (!tau || !b) return invalid("null pointer");
  const int sym = op->g.dim == 2 ? 3 : 6;
  int rc = ensure_spectrum(op, sym);
  if (rc != BRI17_OK) return rc;
  return eigenstress_rhs_batched_async(op, 1, tau, b, op->spec, (cudaStream_t)stream);
}

extern "C" int bri17_eigenstress_to_opposite_strain(bri17_op* op, const void* tau, void* eta,
                                                    void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  {
    const int ts = take_status(op);  // a failure of earlier work on the handle
    if (ts != BRI17_OK) return ts;
  }
  if (!tau || !eta) return invalid("null pointer");
  const int sym = op->g.dim == 2 ? 3 : 6;
  int rc = ensure_spectrum(op, sym);
  if (rc != BRI17_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (op->precision == BRI17_F64)
    return run_pipeline<double, kModeSolve>(op, op->tab64, (const double*)tau, (double*)eta, 1,
                                            op->spec, nullptr, st);
  return run_pipeline<float, kModeSolve>(op, op->tab32, (const float*)tau, (float*)eta, 1,
                                         op->spec, nullptr, st);
}

extern "C" int bri17_op_fused_form(const bri17_op* op, int* form) {
  if (!op || !form) return invalid("null pointer");
  *form = op->float_pair ? op->fused_form_df : op->fused_form;
  return BRI17_OK;
}

extern "C" int bri17_op_set_fused_form(bri17_op* op, int form) {
  if (!op) return invalid("null handle");
  if (form < 0 || form > 3) return invalid("form must be 0, 1, 2 or 3");
  if (op->float_pair)
    op->fused_form_df = form == 2 ? 2 : 1;  // float pairs: staged or TMA-staged
  else
    op->fused_form = form;
  return BRI17_OK;
}

extern "C" int bri17_wait_timeouts(int* count) {
  if (!count) return invalid("null pointer");
  int a = 0, b = 0;
  cudaError_t e = tma_wait_timeouts_f32(&a);
  if (e == cudaSuccess) e = tma_wait_timeouts_df(&b);
  if (e != cudaSuccess) return cuda_fail(e, "reading the wait-timeout count");
  *count = a + b;
  return BRI17_OK;
}

extern "C" int bri17_op_sync_status(bri17_op* op, void* stream) {
  if (!op) return invalid("null handle");
  {
    const int dc = check_device(op);
    if (dc != BRI17_OK) return dc;
  }
  BRI17_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return take_status(op);
}

extern "C" int bri17_set_wait_limit_ns(uint64_t ns) {
  cudaError_t e = tma_set_wait_limit_f32(ns);
  if (e == cudaSuccess) e = tma_set_wait_limit_df(ns);
  if (e != cudaSuccess) return cuda_fail(e, "setting the device wait limit");
  return BRI17_OK;
}

extern "C" int bri17_op_set_pass_timing(bri17_op* op, int enable) {
  if (!op) return invalid("null handle");
  if (enable && !op->timing) op->timing = new PassTiming();
  if (!enable && op->timing) {
    delete reinterpret_cast<PassTiming*>(op->timing);
    op->timing = nullptr;
  }
  return BRI17_OK;
}

extern "C" int bri17_op_pass_times(bri17_op* op, double* ms, int64_t* launches,
                                   int max_passes, int* npasses) {
  if (!op) return invalid("null handle");
  PassTiming* t = reinterpret_cast<PassTiming*>(op->timing);
  if (npasses) *npasses = kNumPasses;
  if (!t) return invalid("pass timing is not enabled");
  t->harvest();
  for (int i = 0; i < kNumPasses && i < max_passes; i++) {
    if (ms) ms[i] = t->ms[i];
    if (launches) launches[i] = t->n[i];
    t->ms[i] = 0;
    t->n[i] = 0;
  }
  return BRI17_OK;
}

extern "C" const char* bri17_pass_name(int pass) {
  static const char* names[kNumPasses] = {"rows_r2c", "axis_c2c_fwd", "axis0_fused",
                                          "axis_c2c_inv", "rows_c2r"};
  return pass >= 0 && pass < kNumPasses ? names[pass] : "unknown";
}
