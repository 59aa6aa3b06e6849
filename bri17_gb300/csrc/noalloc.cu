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
// loads this library holds until the process exits.  A small kernel writes
// the tables into that array on the caller's stream, so a call makes no
// host-to-device copy and returns without waiting for the GPU.
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

std::mutex g_mu;  // guards g_scratch_addr

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

// Device pointers of the FP64 tables inside the scratch array at `dev`, in
// the allocating operator's layout: per axis the twiddles, the half-angle
// unit vectors, then phi, chi, psi, cos(alpha), sin(alpha) N / L.
void table_layout(const int* n, int dim, unsigned char* dev, Tables<double>* tab) {
  memset(tab, 0, sizeof(*tab));
  size_t off = 0;
  for (int i = 0; i < dim; i++) {
    const int m = n[i];
    tab->tw[i] = reinterpret_cast<const double2*>(dev + off);
    off = a16(off + m * sizeof(double2));
    tab->ea[i] = reinterpret_cast<const double2*>(dev + off);
    off = a16(off + m * sizeof(double2));
    const double** d5[5] = {&tab->kphi[i], &tab->kchi[i], &tab->kpsi[i], &tab->bc[i],
                            &tab->bs[i]};
    for (int j = 0; j < 5; j++) {
      *d5[j] = reinterpret_cast<const double*>(dev + off);
      off = a16(off + m * sizeof(double));
    }
  }
}

struct TableArgs {
  Tables<double> tab;
  int dim;
  int n[3];
  double L[3];
};

// Writes the tables on the device, one thread per (axis, k), so that the
// call needs no host buffer and no host-to-device copy.  The values are
// those of the allocating operator's tables to within rounding: phi, chi,
// psi and the half-angle factors follow Hooke::modal_stiffness and
// Hooke::modal_strain_displacement (include/bri17/bri17.hpp:217-224,
// :258-264); the twiddles exp(-2 pi i k / n) come from sincospi, whose
// argument 2k/n carries the only rounding.
__global__ void noalloc_fill_tables(TableArgs a) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int i = 0;
  while (i < a.dim && t >= a.n[i]) t -= a.n[i++];
  if (i >= a.dim) return;
  const int m = a.n[i], k = t;
  const double h = a.L[i] / m;
  double s, c;
  sincospi(2.0 * k / m, &s, &c);
  const_cast<double2*>(a.tab.tw[i])[k] = make_double2(c, -s);
  const double beta = 2 * kPiNA * k / m;
  const double cb = cos(beta);
  const_cast<double*>(a.tab.kphi[i])[k] = 2 * (1 - cb) / h / h;
  const_cast<double*>(a.tab.kchi[i])[k] = (2 + cb) / 3;
  const_cast<double*>(a.tab.kpsi[i])[k] = sin(beta) / h;
  const double alpha = kPiNA * k / m;
  const double ca = cos(alpha), sa = sin(alpha);
  const_cast<double*>(a.tab.bc[i])[k] = ca;
  const_cast<double*>(a.tab.bs[i])[k] = sa * m / a.L[i];
  const_cast<double2*>(a.tab.ea[i])[k] = make_double2(ca, sa);
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
  if (need > kNoAllocScratchBytes)
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
  unsigned char* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      // Once per device, with that device current: the device address of the
      // scratch array.
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
      g_scratch_addr[dev] = p;
    }
    scratch = static_cast<unsigned char*>(g_scratch_addr[dev]);
  }
  TableArgs ta;
  table_layout(g.n, dim, scratch, &ta.tab);
  view.tab64 = ta.tab;
  ta.dim = dim;
  int total = 0;
  for (int i = 0; i < 3; i++) {
    ta.n[i] = g.n[i];
    ta.L[i] = view.L[i];
    if (i < dim) total += g.n[i];
  }
  cudaStream_t st = (cudaStream_t)stream;
  noalloc_fill_tables<<<(total + 127) / 128, 128, 0, st>>>(ta);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "noalloc_fill_tables launch");
  return apply_stiffness_batched_async(&view, 1, u_dev, f_dev, scratch + spec_off, nullptr, st);
}
