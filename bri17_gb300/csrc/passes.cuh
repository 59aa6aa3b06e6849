// passes.cuh -- the FFT passes of the periodic stiffness operator.
//
// The reference applies K as DIM complex-to-complex forward DFTs, a per-mode
// K(k) u(k) loop and DIM backward DFTs (tests/test_bri17.cpp:56-107).  Here
// the fields are real, so the last (contiguous) axis uses a real-to-complex
// transform and only the half spectrum k[dim-1] in [0, n/2] is stored:
//
//   u (real, SoA) --rows_r2c--> S[c][k0][k1][k2'] --axis_c2c (axis 1, 3D)-->
//   --axis0_fused: forward DFT along axis 0, per-mode operator, inverse DFT-->
//   --axis_c2c inverse (axis 1, 3D)--> --rows_c2r--> f (real, SoA)
//
// The per-mode operator is generated in registers from per-axis tables
// (never stored), and the normalisation |h|/|N| of compute_Ku
// (tests/test_bri17.cpp:93-106) is folded into it.  K(-k) = K(k) for the
// reference's K (psi flips sign in pairs, include/bri17/bri17.hpp:281-285),
// so the product of a Hermitian spectrum stays Hermitian and the C2R
// transform returns the real part the reference extracts at :140-145.
#pragma once

#include "common.cuh"
#include "pdl.cuh"

namespace bri17gb {

constexpr int kThreads = 256;

// kModeSolve: eigenstress -> opposite strain, the field form of
// Hooke::modal_eigenstress_to_opposite_strain (include/bri17/bri17.hpp:308-355).
enum FusedMode { kModeStiffness = 0, kModeStrain = 1, kModeRhs = 2, kModeSolve = 3 };

// Optional per-batch-entry mask: a CTA whose work belongs to entry z exits
// at once when flags[z * stride] == 0.  `unit` is the number of CTA work
// units (rows, outer lines) of one entry; null flags = every entry active.
struct BatchMask {
  const int* flags;
  int stride;
  int64_t unit;
  __device__ __forceinline__ bool skip(int64_t first_unit) const {
    return flags && flags[(first_unit / unit) * stride] == 0;
  }
};

struct CgState;

template <typename T>
struct FusedParams {
  Tables<T> tab;
  int n1;           // 3D: cells along axis 1; 2D: unused
  int H;            // half length of the last axis
  T s;              // (lambda + mu) * corr: "scaling" of
                    // include/bri17/bri17.hpp:266 times the normalisation
  T mu;             // mu * corr
  T corr;           // normalisation of strain / rhs modes
  const T* mat;     // optional per-batch (s, mu) pairs, overriding s, mu
  int form;         // power-of-two axis-0 stiffness pass: 0 registers, 1 staged
  int* status;      // the handle's status words (mapped host memory) or null
  // A CG iteration's p.Kp, summed by Parseval in the FP32 TMA-staged
  // stiffness pass (axis0_stiffness_tma with PQ) into `cg` (pq, alpha) with
  // one partial per CTA in cg_part; null outside CG iterations.
  CgState* cg = nullptr;
  double* cg_part = nullptr;
};

// ---------------------------------------------------------------------------
// Last axis, forward: real rows of length n -> n/2+1 complex.
// Even n packs z_j = x_2j + i x_2j+1, transforms length m = n/2 and splits
// X_k = E_k + W_n^k O_k; odd n transforms the full row with zero imaginary.

template <typename T>
__global__ void __launch_bounds__(kThreads)
    rows_r2c(const T* __restrict__ x, cplx<T>* __restrict__ X, int64_t nrows,
             int n, int H, AxisPlan pm, const cplx<T>* __restrict__ tw_g,
             int rows_per_cta, int pitch, BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* a = tw + n;
  cplx<T>* b = a + rows_per_cta * pitch;
  const bool even = (n % 2) == 0;
  const int m = even ? n / 2 : n;
  const int64_t row0 = (int64_t)blockIdx.x * rows_per_cta;
  const int nr = (int)min((int64_t)rows_per_cta, nrows - row0);
  pdl_launch_dependents<T>();
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = tw_g[t];
  pdl_wait();
  if (mask.skip(row0)) return;
  if (even) {
    const cplx<T>* xc = reinterpret_cast<const cplx<T>*>(x) + row0 * m;
    for (int f = threadIdx.x; f < nr * m; f += blockDim.x) {
      const int r = f / m;
      a[r * pitch + (f - r * m)] = xc[f];
    }
  } else {
    const T* xr = x + row0 * n;
    for (int f = threadIdx.x; f < nr * n; f += blockDim.x) {
      const int r = f / n;
      a[r * pitch + (f - r * n)] = mk<T>(xr[f], T(0));
    }
  }
  __syncthreads();
  fft_lines<T, false>(a, b, nr, pitch, pm, tw, even ? 2 : 1);
  cplx<T>* out = X + row0 * H;
  for (int f = threadIdx.x; f < nr * H; f += blockDim.x) {
    const int r = f / H;
    const int k = f - r * H;
    cplx<T> v;
    if (even) {
      const cplx<T> zk = a[r * pitch + (k == m ? 0 : k)];
      const cplx<T> zm = a[r * pitch + (k == 0 ? 0 : m - k)];
      const T h = T(0.5);
      const cplx<T> e = mk<T>(h * (zk.x + zm.x), h * (zk.y - zm.y));
      const cplx<T> o = mk<T>(h * (zk.y + zm.y), h * (zm.x - zk.x));
      v = cadd<T>(e, cmul<T>(tw[k], o));
    } else {
      v = a[r * pitch + k];
    }
    out[f] = v;
  }
}

// Last axis, inverse: n/2+1 complex -> real rows of length n (unnormalised).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    rows_c2r(const cplx<T>* __restrict__ X, T* __restrict__ x, int64_t nrows,
             int n, int H, AxisPlan pm, const cplx<T>* __restrict__ tw_g,
             int rows_per_cta, int pitch, BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* a = tw + n;
  cplx<T>* b = a + rows_per_cta * pitch;
  const bool even = (n % 2) == 0;
  const int m = even ? n / 2 : n;
  const int64_t row0 = (int64_t)blockIdx.x * rows_per_cta;
  const int nr = (int)min((int64_t)rows_per_cta, nrows - row0);
  pdl_launch_dependents<T>();
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = tw_g[t];
  __syncthreads();
  pdl_wait();
  if (mask.skip(row0)) return;
  const cplx<T>* in = X + row0 * H;
  if (even) {
    for (int f = threadIdx.x; f < nr * m; f += blockDim.x) {
      const int r = f / m;
      const int k = f - r * m;
      const cplx<T> xk = in[r * H + k];
      const cplx<T> xm = in[r * H + (m - k)];
      // A = X_k + conj(X_{m-k});  Bv = (X_k - conj(X_{m-k})) W_n^{-k};
      // Z_k = A + i Bv.
      const cplx<T> A = mk<T>(xk.x + xm.x, xk.y - xm.y);
      const cplx<T> D = mk<T>(xk.x - xm.x, xk.y + xm.y);
      const cplx<T> Bv = cmulc<T>(D, tw[k]);
      a[r * pitch + k] = mk<T>(A.x - Bv.y, A.y + Bv.x);
    }
  } else {
    for (int f = threadIdx.x; f < nr * n; f += blockDim.x) {
      const int r = f / n;
      const int k = f - r * n;
      cplx<T> v;
      if (k < H) {
        v = in[r * H + k];
      } else {
        v = in[r * H + (n - k)];
        v.y = -v.y;
      }
      a[r * pitch + k] = v;
    }
  }
  __syncthreads();
  fft_lines<T, true>(a, b, nr, pitch, pm, tw, even ? 2 : 1);
  if (even) {
    cplx<T>* xc = reinterpret_cast<cplx<T>*>(x) + row0 * m;
    for (int f = threadIdx.x; f < nr * m; f += blockDim.x) {
      const int r = f / m;
      xc[f] = a[r * pitch + (f - r * m)];
    }
  } else {
    T* xr = x + row0 * n;
    for (int f = threadIdx.x; f < nr * n; f += blockDim.x) {
      const int r = f / n;
      xr[f] = a[r * pitch + (f - r * n)].x;
    }
  }
}

// ---------------------------------------------------------------------------
// A middle axis: complex array [A][n][B]; lines along n, a CTA takes TB
// consecutive inner indices b of one outer index a (coalesced loads of TB
// contiguous complex values per element).

template <typename T, bool INV>
__global__ void __launch_bounds__(kThreads)
    axis_c2c(cplx<T>* __restrict__ X, int n, int64_t B, int TB, int pitch,
             AxisPlan p, const cplx<T>* __restrict__ tw_g, BatchMask mask) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* a = tw + n;
  cplx<T>* b = a + TB * pitch;
  const int64_t b0 = (int64_t)blockIdx.x * TB;
  const int nb = (int)min((int64_t)TB, B - b0);
  cplx<T>* base = X + (int64_t)blockIdx.y * n * B + b0;
  pdl_launch_dependents<T>();
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = tw_g[t];
  pdl_wait();
  if (mask.skip(blockIdx.y)) return;
  for (int f = threadIdx.x; f < n * nb; f += blockDim.x) {
    const int i = f / nb;
    const int tb = f - i * nb;
    a[tb * pitch + i] = base[(int64_t)i * B + tb];
  }
  __syncthreads();
  fft_lines<T, INV>(a, b, nb, pitch, p, tw, 1);
  for (int f = threadIdx.x; f < n * nb; f += blockDim.x) {
    const int i = f / nb;
    const int tb = f - i * nb;
    base[(int64_t)i * B + tb] = a[tb * pitch + i];
  }
}

// ---------------------------------------------------------------------------
// Per-mode operators.

// 3D modal stiffness times u, generated from the per-axis tables.  Entry
// formulas of Hooke::modal_stiffness (include/bri17/bri17.hpp:276-288) with
// s = scaling * corr and mu = mu * corr.
template <typename T>
__device__ __forceinline__ void stiffness3(T phi0, T chi0, T psi0, T phi1,
                                           T chi1, T psi1, T phi2, T chi2,
                                           T psi2, T s, T mu, cplx<T>* u) {
  const T H00 = phi0 * chi1 * chi2;
  const T H11 = chi0 * phi1 * chi2;
  const T H22 = chi0 * chi1 * phi2;
  const T Kd = mu * (H00 + H11 + H22);
  const T K00 = s * H00 + Kd;
  const T K11 = s * H11 + Kd;
  const T K22 = s * H22 + Kd;
  const T K01 = s * psi0 * psi1 * chi2;
  const T K02 = s * psi0 * chi1 * psi2;
  const T K12 = s * chi0 * psi1 * psi2;
  const cplx<T> u0 = u[0], u1 = u[1], u2 = u[2];
  u[0] = mk<T>(K00 * u0.x + K01 * u1.x + K02 * u2.x,
               K00 * u0.y + K01 * u1.y + K02 * u2.y);
  u[1] = mk<T>(K01 * u0.x + K11 * u1.x + K12 * u2.x,
               K01 * u0.y + K11 * u1.y + K12 * u2.y);
  u[2] = mk<T>(K02 * u0.x + K12 * u1.x + K22 * u2.x,
               K02 * u0.y + K12 * u1.y + K22 * u2.y);
}

// 2D: include/bri17/bri17.hpp:267-274.
template <typename T>
__device__ __forceinline__ void stiffness2(T phi0, T chi0, T psi0, T phi1,
                                           T chi1, T psi1, T s, T mu,
                                           cplx<T>* u) {
  const T H00 = phi0 * chi1;
  const T H11 = chi0 * phi1;
  const T Kd = mu * (H00 + H11);
  const T K00 = s * H00 + Kd;
  const T K11 = s * H11 + Kd;
  const T K01 = s * psi0 * psi1;
  const cplx<T> u0 = u[0], u1 = u[1];
  u[0] = mk<T>(K00 * u0.x + K01 * u1.x, K00 * u0.y + K01 * u1.y);
  u[1] = mk<T>(K01 * u0.x + K11 * u1.x, K01 * u0.y + K11 * u1.y);
}

// The real symmetric K(k) itself (same products as stiffness3/stiffness2),
// row-major DIM x DIM.
template <typename T, int DIM>
__device__ __forceinline__ void stiffness_matrix(const T* phi, const T* chi, const T* psi, T s,
                                                 T mu, T* K) {
  if constexpr (DIM == 3) {
    const T H00 = phi[0] * chi[1] * chi[2];
    const T H11 = chi[0] * phi[1] * chi[2];
    const T H22 = chi[0] * chi[1] * phi[2];
    const T Kd = mu * (H00 + H11 + H22);
    K[0] = s * H00 + Kd;
    K[4] = s * H11 + Kd;
    K[8] = s * H22 + Kd;
    K[1] = K[3] = s * psi[0] * psi[1] * chi[2];
    K[2] = K[6] = s * psi[0] * chi[1] * psi[2];
    K[5] = K[7] = s * chi[0] * psi[1] * psi[2];
  } else {
    const T H00 = phi[0] * chi[1];
    const T H11 = chi[0] * phi[1];
    const T Kd = mu * (H00 + H11);
    K[0] = s * H00 + Kd;
    K[3] = s * H11 + Kd;
    K[1] = K[2] = s * psi[0] * psi[1];
  }
}

// Solves K u = r for a real symmetric positive definite K (DIM x DIM,
// row-major) and complex r, by LDL^T (the reference's Eigen LLT,
// include/bri17/bri17.hpp:341, in a square-root-free form).
template <typename T, int DIM>
__device__ __forceinline__ void spd_solve(const T* K, const cplx<T>* r, cplx<T>* u) {
  T L[DIM][DIM], D[DIM];
#pragma unroll
  for (int j = 0; j < DIM; j++) {
    T d = K[j * DIM + j];
#pragma unroll
    for (int p = 0; p < j; p++) d -= L[j][p] * L[j][p] * D[p];
    D[j] = d;
#pragma unroll
    for (int i = j + 1; i < DIM; i++) {
      T v = K[i * DIM + j];
#pragma unroll
      for (int p = 0; p < j; p++) v -= L[i][p] * L[j][p] * D[p];
      L[i][j] = v / d;
    }
  }
  cplx<T> y[DIM];
#pragma unroll
  for (int i = 0; i < DIM; i++) {
    cplx<T> v = r[i];
#pragma unroll
    for (int p = 0; p < i; p++) v = csub<T>(v, cscale<T>(y[p], L[i][p]));
    y[i] = v;
  }
#pragma unroll
  for (int i = DIM - 1; i >= 0; i--) {
    cplx<T> v = cscale<T>(y[i], T(1) / D[i]);
#pragma unroll
    for (int p = i + 1; p < DIM; p++) v = csub<T>(v, cscale<T>(u[p], L[p][i]));
    u[i] = v;
  }
}

// Modal strain-displacement vector (include/bri17/bri17.hpp:212-236):
// B_i = 2 i e^{i sum alpha} s_i prod_{j != i} c_j.
template <typename T, int DIM>
__device__ __forceinline__ void bvec(const T* c, const T* s, cplx<T> e,
                                     cplx<T>* B) {
  const cplx<T> pre = mk<T>(-2 * e.y, 2 * e.x);
  if constexpr (DIM == 2) {
    B[0] = cscale<T>(pre, s[0] * c[1]);
    B[1] = cscale<T>(pre, c[0] * s[1]);
  } else {
    B[0] = cscale<T>(pre, s[0] * c[1] * c[2]);
    B[1] = cscale<T>(pre, c[0] * s[1] * c[2]);
    B[2] = cscale<T>(pre, c[0] * c[1] * s[2]);
  }
}

// Mandel pair (i, j) of strain component q: (xx,yy,xy) in 2D,
// (xx,yy,zz,yz,zx,xy) in 3D (include/bri17/bri17.hpp:324-332, :343-353).
template <int DIM>
__device__ __forceinline__ void mandel_pair(int q, int& i, int& j) {
  if constexpr (DIM == 2) {
    const int I[3] = {0, 1, 0}, J[3] = {0, 1, 1};
    i = I[q];
    j = J[q];
  } else {
    const int I[6] = {0, 1, 2, 1, 2, 0}, J[6] = {0, 1, 2, 2, 0, 1};
    i = I[q];
    j = J[q];
  }
}

// ---------------------------------------------------------------------------
// Axis 0, fused: forward DFT of the cin input components along axis 0, the
// per-mode operator, inverse DFT of the cout output components, in place.
// Spectrum component c of batch entry z at X + z*bstride + c*cstride, line b
// of axis-0 element k0 at k0*P + b.  Line b encodes (k1, k2') = (b / H,
// b % H) in 3D and k1' = b in 2D.

template <typename T, int DIM, int MODE>
__global__ void __launch_bounds__(kThreads)
    axis0_fused(cplx<T>* __restrict__ X, int n0, int64_t P, int64_t cstride,
                int64_t bstride, int TB, int pitch, AxisPlan p0,
                FusedParams<T> fp, BatchMask mask) {
  constexpr int SYM = DIM == 2 ? 3 : 6;
  constexpr int CIN = (MODE == kModeRhs || MODE == kModeSolve) ? SYM : DIM;
  constexpr int COUT = (MODE == kModeStrain || MODE == kModeSolve) ? SYM : DIM;
  constexpr int CMAX = CIN > COUT ? CIN : COUT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n0;  // CMAX + 1 buffers of TB * pitch
  const int64_t b0 = (int64_t)blockIdx.x * TB;
  const int nb = (int)min((int64_t)TB, P - b0);
  cplx<T>* base = X + (int64_t)blockIdx.y * bstride + b0;
  pdl_launch_dependents<T>();
  for (int t = threadIdx.x; t < n0; t += blockDim.x) tw[t] = fp.tab.tw[0][t];
  pdl_wait();
  if (mask.skip(blockIdx.y)) return;
  T s = fp.s, mu = fp.mu;
  if (fp.mat) {
    s = fp.mat[2 * blockIdx.y];
    mu = fp.mat[2 * blockIdx.y + 1];
  }
  for (int c = 0; c < CIN; c++) {
    cplx<T>* a = buf + c * TB * pitch;
    const cplx<T>* src = base + c * cstride;
    for (int f = threadIdx.x; f < n0 * nb; f += blockDim.x) {
      const int i = f / nb;
      const int tb = f - i * nb;
      a[tb * pitch + i] = src[(int64_t)i * P + tb];
    }
  }
  __syncthreads();
  cplx<T>* scratch = buf + CMAX * TB * pitch;
  for (int c = 0; c < CIN; c++)
    fft_lines<T, false>(buf + c * TB * pitch, scratch, nb, pitch, p0, tw, 1);
  // Per-mode operator.
  for (int f = threadIdx.x; f < n0 * nb; f += blockDim.x) {
    const int tb = f / n0;
    const int k0 = f - tb * n0;
    const int64_t b = b0 + tb;
    int k1, k2 = 0;
    if constexpr (DIM == 3) {
      k1 = (int)(b / fp.H);
      k2 = (int)(b - (int64_t)k1 * fp.H);
    } else {
      k1 = (int)b;
    }
    const int off = tb * pitch + k0;
    if constexpr (MODE == kModeStiffness) {
      cplx<T> u[DIM];
#pragma unroll
      for (int c = 0; c < DIM; c++) u[c] = buf[c * TB * pitch + off];
      if constexpr (DIM == 3) {
        stiffness3<T>(fp.tab.kphi[0][k0], fp.tab.kchi[0][k0], fp.tab.kpsi[0][k0],
                      __ldg(fp.tab.kphi[1] + k1), __ldg(fp.tab.kchi[1] + k1),
                      __ldg(fp.tab.kpsi[1] + k1), __ldg(fp.tab.kphi[2] + k2),
                      __ldg(fp.tab.kchi[2] + k2), __ldg(fp.tab.kpsi[2] + k2), s,
                      mu, u);
      } else {
        stiffness2<T>(fp.tab.kphi[0][k0], fp.tab.kchi[0][k0], fp.tab.kpsi[0][k0],
                      __ldg(fp.tab.kphi[1] + k1), __ldg(fp.tab.kchi[1] + k1),
                      __ldg(fp.tab.kpsi[1] + k1), s, mu, u);
      }
#pragma unroll
      for (int c = 0; c < DIM; c++) buf[c * TB * pitch + off] = u[c];
    } else {
      const int kk[3] = {k0, k1, k2};
      T cc[DIM], ss[DIM];
      cplx<T> e = mk<T>(T(1), T(0));
#pragma unroll
      for (int d = 0; d < DIM; d++) {
        cc[d] = __ldg(fp.tab.bc[d] + kk[d]);
        ss[d] = __ldg(fp.tab.bs[d] + kk[d]);
        e = cmul<T>(e, fp.tab.ea[d][kk[d]]);
      }
      cplx<T> B[DIM];
      bvec<T, DIM>(cc, ss, e, B);
      if constexpr (MODE == kModeSolve) {
        // eta_hat = corr * sym(B (x) u), u = K^-1 (tau_mat . conj(B)); k = 0
        // gives 0 (include/bri17/bri17.hpp:333-354).
        cplx<T> tau[SYM];
#pragma unroll
        for (int q = 0; q < SYM; q++) tau[q] = buf[q * TB * pitch + off];
        const T ir2 = T(0.7071067811865475244008443621048490392848);
        const T r2 = T(1.414213562373095048801688724209698079);
        cplx<T> rhs[DIM];
#pragma unroll
        for (int d = 0; d < DIM; d++) rhs[d] = mk<T>(T(0), T(0));
#pragma unroll
        for (int q = 0; q < SYM; q++) {
          int i, j;
          mandel_pair<DIM>(q, i, j);
          if (i == j) {
            rhs[i] = cadd<T>(rhs[i], cmulc<T>(tau[q], B[i]));
          } else {
            const cplx<T> t = cscale<T>(tau[q], ir2);
            rhs[i] = cadd<T>(rhs[i], cmulc<T>(t, B[j]));
            rhs[j] = cadd<T>(rhs[j], cmulc<T>(t, B[i]));
          }
        }
        const bool null_frequency = k0 == 0 && k1 == 0 && k2 == 0;
        T phi[DIM], chi[DIM], psi[DIM], K[DIM * DIM];
#pragma unroll
        for (int d = 0; d < DIM; d++) {
          phi[d] = __ldg(fp.tab.kphi[d] + kk[d]);
          chi[d] = __ldg(fp.tab.kchi[d] + kk[d]);
          psi[d] = __ldg(fp.tab.kpsi[d] + kk[d]);
        }
        stiffness_matrix<T, DIM>(phi, chi, psi, s, mu, K);
        cplx<T> u[DIM];
        spd_solve<T, DIM>(K, rhs, u);
#pragma unroll
        for (int q = 0; q < SYM; q++) {
          int i, j;
          mandel_pair<DIM>(q, i, j);
          cplx<T> v = cadd<T>(cmul<T>(B[i], u[j]), cmul<T>(u[i], B[j]));
          const T w = (i == j ? T(0.5) : T(0.5) * r2) * fp.corr;
          buf[q * TB * pitch + off] =
              null_frequency ? mk<T>(T(0), T(0)) : cscale<T>(v, w);
        }
      } else if constexpr (MODE == kModeStrain) {
        // eps_hat = corr * sym(u (x) B), sqrt(2) on the shears
        // (tests/test_bri17.cpp:223-230).
        cplx<T> u[DIM];
#pragma unroll
        for (int c = 0; c < DIM; c++) u[c] = buf[c * TB * pitch + off];
        const T r2 = T(1.414213562373095048801688724209698079);
#pragma unroll
        for (int q = 0; q < SYM; q++) {
          int i, j;
          mandel_pair<DIM>(q, i, j);
          cplx<T> v = cadd<T>(cmul<T>(B[i], u[j]), cmul<T>(u[i], B[j]));
          const T w = (i == j ? T(0.5) : T(0.5) * r2) * fp.corr;
          buf[q * TB * pitch + off] = cscale<T>(v, w);
        }
      } else {
        // b_hat = -corr * tau_mat . conj(B) (include/bri17/bri17.hpp:340).
        cplx<T> tau[SYM];
#pragma unroll
        for (int q = 0; q < SYM; q++) tau[q] = buf[q * TB * pitch + off];
        const T ir2 = T(0.7071067811865475244008443621048490392848);
        cplx<T> out[DIM];
#pragma unroll
        for (int d = 0; d < DIM; d++) out[d] = mk<T>(T(0), T(0));
#pragma unroll
        for (int q = 0; q < SYM; q++) {
          int i, j;
          mandel_pair<DIM>(q, i, j);
          if (i == j) {
            out[i] = cadd<T>(out[i], cmulc<T>(tau[q], B[i]));
          } else {
            const cplx<T> t = cscale<T>(tau[q], ir2);
            out[i] = cadd<T>(out[i], cmulc<T>(t, B[j]));
            out[j] = cadd<T>(out[j], cmulc<T>(t, B[i]));
          }
        }
#pragma unroll
        for (int d = 0; d < DIM; d++)
          buf[d * TB * pitch + off] = cscale<T>(out[d], -fp.corr);
      }
    }
  }
  __syncthreads();
  for (int c = 0; c < COUT; c++)
    fft_lines<T, true>(buf + c * TB * pitch, scratch, nb, pitch, p0, tw, 1);
  for (int c = 0; c < COUT; c++) {
    const cplx<T>* a = buf + c * TB * pitch;
    cplx<T>* dst = base + c * cstride;
    for (int f = threadIdx.x; f < n0 * nb; f += blockDim.x) {
      const int i = f / nb;
      const int tb = f - i * nb;
      dst[(int64_t)i * P + tb] = a[tb * pitch + i];
    }
  }
}

}  // namespace bri17gb
