// common.cuh -- shared host/device declarations of the bri17 GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>

#include "../../include/bri17_gb300.h"
#include "fft.cuh"
#include "fft8.cuh"

namespace bri17gb {

// Per-thread last-error text behind bri17_last_error().
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define BRI17_CUDA_TRY(expr)                           \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
  } while (0)

// Device tables of one operator, in scalar type T.  For axis i of length n:
//   tw[i][t]   = exp(-2 pi i t / n), t in [0, n)           (FFT twiddles)
//   kphi/kchi/kpsi[i][k] = phi, chi, psi of Hooke::modal_stiffness
//                (include/bri17/bri17.hpp:258-264), k in [0, n)
//   bc[i][k] = cos(alpha), bs[i][k] = sin(alpha) N / L, ea[i][k] =
//                (cos alpha, sin alpha), alpha = pi k / N, the factors of
//                Hooke::modal_strain_displacement (:217-224)
template <typename T>
struct Tables {
  const cplx<T>* tw[3];
  const T* kphi[3];
  const T* kchi[3];
  const T* kpsi[3];
  const T* bc[3];
  const T* bs[3];
  const cplx<T>* ea[3];
};

// Geometry of one operator's real fields and half spectrum.
struct Geometry {
  int dim;
  int n[3];        // cells per axis (axis dim-1 is the contiguous one)
  int H;           // n[dim-1] / 2 + 1
  int64_t size;    // nodes
  int64_t P;       // spectrum lines per component along axis 0
  int64_t cspec;   // complex spectrum entries per component (n[0] * P)
  AxisPlan plan_row;  // last axis: length n/2 (even n) or n (odd n)
  AxisPlan plan[3];   // full-length plans of each axis
  // Register-resident plans for power-of-two lengths (fft8.cuh); a pass
  // uses them when its flag is set, else the generic engine.
  Plan8 p8_row;       // last axis, length n/2
  Plan8 p8[3];
  bool use_p8_row;
  bool use_p8[3];
  // Lengths 3 * 2^k: the compile-time twelve-element engine (CtEng3) where
  // it has an instance, else the generic engine.
  bool use_ct3_row;
  bool use_ct3[3];
};

inline bool is_3pow2(int n) { return n > 0 && n % 3 == 0 && is_pow2(n / 3) && n / 3 >= 8; }

// Fill the register-resident plans of a geometry whose n, dim are set.
inline void set_p8_plans(Geometry* g) {
  const int nl = g->n[g->dim - 1];
  g->use_p8_row = (nl % 2 == 0) && make_plan8(nl / 2, &g->p8_row);
  g->use_ct3_row = (nl % 2 == 0) && is_3pow2(nl / 2);
  for (int i = 0; i < 3; i++) {
    g->use_p8[i] = i < g->dim && make_plan8(g->n[i], &g->p8[i]);
    g->use_ct3[i] = i < g->dim && is_3pow2(g->n[i]);
  }
}

bool make_plan(int n, AxisPlan* p);

// Runs f() once for each CUDA device it is called with current.  Kernel
// attributes (the dynamic shared-memory limit among them) belong to a
// device, so they are set again on every device a process uses.  `done`
// holds one bit per device ordinal below 64; higher ordinals run f() on
// every call.
template <typename F>
void once_per_device(std::atomic<unsigned long long>* done, F&& f) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (dev < 0 || dev >= 64) {
    f();
    return;
  }
  const unsigned long long bit = 1ull << dev;
  if (done->load(std::memory_order_acquire) & bit) return;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (done->load(std::memory_order_relaxed) & bit) return;
  f();
  done->fetch_or(bit, std::memory_order_release);
}

}  // namespace bri17gb
