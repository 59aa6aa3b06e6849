// noalloc.cu -- f = K u for callers that cannot allocate device memory.
//
// bri17_apply_stiffness allocates its half-spectrum scratch and tables when
// the handle is created (cudaMalloc).  Some callers cannot do that: a plugin
// inside a host application that owns every device allocation and forbids
// its plugins to call cudaMalloc, code that must run under a fixed device
// memory budget decided before it starts, or a caller that must not let
// cudaMalloc/cudaFree synchronise the device in the middle of its own work.
// bri17_apply_stiffness_noalloc serves them: it takes the same inputs and
// outputs, allocates nothing, and keeps its scratch (per-axis tables + the
// half spectrum) in the fixed-size device array below, which every GPU that
// loads this library holds until the process exits.
#include <math.h>
#include <string.h>

#include <mutex>

#include "op.cuh"

namespace bri17gb {
namespace {

// Maximum scratch of the no-alloc entry point: 64 MiB per device.  It holds
// the tables (72 bytes per grid point of each axis) and the FP64 half
// spectrum (dim * n0 * n1 * (n2/2+1) * 16 bytes), which covers 128^3.
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device.  The symbol's name in host
// code is a host-side stand-in, not a device address, so every kernel gets
// the address that cudaGetSymbolAddress returned on that device.
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices];

// Host staging of the tables (3 axes x 1024 points x 72 bytes + padding).
constexpr size_t kTableStageBytes = 256 * 1024;
alignas(16) unsigned char g_table_stage[kTableStageBytes];

std::mutex g_mu;  // guards g_scratch_addr and g_table_stage

constexpr double kPiNA = 3.141592653589793238462643383279502884;

size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

// Same radix factorisation as make_plan, without heap allocation.
bool plan_fixed(int n, AxisPlan* p) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  if (n < 1) return false;
  int r[kMaxStages + 8];
  int nr = 0, e = 0, m = n;
  while (m % 2 == 0) {
    m /= 2;
    e++;
  }
  const int q = e / 4, rem = e % 4;
  for (int i = 0; i < q; i++) r[nr++] = 16;
  if (rem == 1) {
    if (q >= 1) {
      r[nr - 1] = 8;
      r[nr++] = 4;
    } else {
      r[nr++] = 2;
    }
  } else if (rem == 2) {
    r[nr++] = 4;
  } else if (rem == 3) {
    r[nr++] = 8;
  }
  for (int f = 3; m > 1; f += 2) {
    while (m % f == 0) {
      if (f > kMaxGenericRadix || nr >= kMaxStages) return false;
      r[nr++] = f;
      m /= f;
    }
  }
  if (nr > kMaxStages) return false;
  p->nstages = nr;
  for (int i = 0; i < nr; i++) p->radix[i] = r[i];
  return true;
}

// Bytes of the FP64 tables of all axes (layout of fill_tables_fixed).
size_t table_bytes(const int* n, int dim) {
  size_t b = 0;
  for (int i = 0; i < dim; i++) {
    b = a16(b + n[i] * 2 * sizeof(double));
    b = a16(b + n[i] * 2 * sizeof(double));
    for (int j = 0; j < 5; j++) b = a16(b + n[i] * sizeof(double));
  }
  return b;
}

// FP64 tables into `host`, with device pointers into `dev`: the same values
// and layout as the allocating operator's tables.
void fill_tables_fixed(const int* n, const double* L, int dim, unsigned char* host,
                       unsigned char* dev, Tables<double>* tab) {
  const long double pil = 3.141592653589793238462643383279502884L;
  memset(tab, 0, sizeof(*tab));
  size_t off = 0;
  for (int i = 0; i < dim; i++) {
    const int m = n[i];
    const double h = L[i] / m;
    double2* tw = reinterpret_cast<double2*>(host + off);
    tab->tw[i] = reinterpret_cast<const double2*>(dev + off);
    off = a16(off + m * sizeof(double2));
    double2* ea = reinterpret_cast<double2*>(host + off);
    tab->ea[i] = reinterpret_cast<const double2*>(dev + off);
    off = a16(off + m * sizeof(double2));
    double* t5[5];
    const double** d5[5] = {&tab->kphi[i], &tab->kchi[i], &tab->kpsi[i], &tab->bc[i],
                            &tab->bs[i]};
    for (int j = 0; j < 5; j++) {
      t5[j] = reinterpret_cast<double*>(host + off);
      *d5[j] = reinterpret_cast<const double*>(dev + off);
      off = a16(off + m * sizeof(double));
    }
    for (int k = 0; k < m; k++) {
      const long double ang = 2.0L * pil * (long double)k / (long double)m;
      tw[k].x = (double)cosl(ang);
      tw[k].y = (double)-sinl(ang);
      const double beta = 2 * kPiNA * k / m;
      t5[0][k] = 2 * (1 - cos(beta)) / h / h;
      t5[1][k] = (2 + cos(beta)) / 3;
      t5[2][k] = sin(beta) / h;
      const double alpha = kPiNA * k / m;
      t5[3][k] = cos(alpha);
      t5[4][k] = sin(alpha) * m / L[i];
      ea[k].x = cos(alpha);
      ea[k].y = sin(alpha);
    }
  }
}

int fail(int status, const char* msg) {
  set_error(msg);
  return status;
}

}  // namespace
}  // namespace bri17gb

using namespace bri17gb;

extern "C" int bri17_apply_stiffness_noalloc(int dim, const int* shape, const double* L,
                                             double mu, double nu, const double* u_dev,
                                             double* f_dev, void* stream) {
  if (!shape || !L || !u_dev || !f_dev) return fail(BRI17_ERR_INVALID_ARGUMENT, "null pointer");
  if (dim != 2 && dim != 3) return fail(BRI17_ERR_INVALID_ARGUMENT, "dim must be 2 or 3");
  if (!(mu > 0) || !isfinite(mu)) return fail(BRI17_ERR_INVALID_ARGUMENT, "mu must be positive");
  if (!(nu > -1.0 && nu < 0.5)) return fail(BRI17_ERR_INVALID_ARGUMENT, "nu must lie in (-1, 0.5)");
  bri17_op view;
  memset(&view, 0, sizeof(view));
  Geometry& g = view.g;
  g.dim = dim;
  g.size = 1;
  for (int i = 0; i < 3; i++) {
    g.n[i] = i < dim ? shape[i] : 1;
    view.L[i] = i < dim ? L[i] : 1.0;
  }
  for (int i = 0; i < dim; i++) {
    if (shape[i] < 1) return fail(BRI17_ERR_INVALID_ARGUMENT, "shape entries must be >= 1");
    if (!(L[i] > 0) || !isfinite(L[i])) return fail(BRI17_ERR_INVALID_ARGUMENT, "L entries must be positive");
    if (shape[i] > 1024) return fail(BRI17_ERR_UNSUPPORTED_SIZE, "axis length above 1024");
    g.size *= shape[i];
  }
  const int nl = g.n[dim - 1];
  g.H = nl / 2 + 1;
  g.P = dim == 3 ? (int64_t)g.n[1] * g.H : (int64_t)g.H;
  g.cspec = (int64_t)g.n[0] * g.P;
  bool ok = plan_fixed(nl % 2 == 0 ? nl / 2 : nl, &g.plan_row);
  for (int i = 0; i < dim; i++) ok = ok && plan_fixed(g.n[i], &g.plan[i]);
  set_p8_plans(&g);
  if (!ok) return fail(BRI17_ERR_UNSUPPORTED_SIZE, "axis length has a prime factor above 61");
  const size_t tbytes = table_bytes(g.n, dim);
  const size_t spec_off = (tbytes + 255) & ~size_t(255);
  const size_t need = spec_off + (size_t)dim * g.cspec * sizeof(double2);
  if (need > kNoAllocScratchBytes || tbytes > kTableStageBytes)
    return fail(BRI17_ERR_UNSUPPORTED_SIZE,
                "grid too large for the no-alloc entry point: it needs more than its fixed "
                "64 MiB device scratch (tables + FP64 half spectrum); use bri17_apply_stiffness");
  view.mu = mu;
  view.nu = nu;
  view.precision = BRI17_F64;
  double cv = 1.0;
  for (int i = 0; i < dim; i++) cv *= view.L[i] / g.n[i];
  view.cell_volume = cv;
  view.corr = cv / (double)g.size;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(BRI17_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    // Once per device, with that device current: the device address of the
    // scratch array.
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_addr[dev] = p;
  }
  unsigned char* scratch = static_cast<unsigned char*>(g_scratch_addr[dev]);
  fill_tables_fixed(g.n, view.L, dim, g_table_stage, scratch, &view.tab64);
  cudaStream_t st = (cudaStream_t)stream;
  // Pageable source: the call returns once the staging buffer is consumed,
  // so g_table_stage may be refilled by the next call.
  e = cudaMemcpyAsync(scratch, g_table_stage, tbytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(tables)");
  return apply_stiffness_batched_async(&view, 1, u_dev, f_dev, scratch + spec_off, nullptr, st);
}
