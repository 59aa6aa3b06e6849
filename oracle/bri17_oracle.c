/*
 * bri17_oracle.c -- CPU restatement of the reference algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  Nothing in the product path (bri17_gb300/, include/) links or calls it.
 *
 * Every function restates one piece of sbrisard/bri17 and cites the file and
 * lines it follows.  The per-mode functions keep the reference's operation
 * order so that, compiled with -ffp-contract=off, they agree bit for bit with
 * the reference header compiled the same way (checked in tests/test_oracle.py
 * against oracle/_ref and against the committed fixtures).
 *
 * Complex arrays are interleaved (re, im) doubles.  Spectra and fields use the
 * reference's SoA layout: component c of node n at index c * size + n, nodes
 * in row-major order, last axis fastest (include/bri17/bri17.hpp:78-93,
 * tests/test_bri17.cpp:66-67).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* std::numbers::pi_v<double> and std::numbers::sqrt2_v<double>. */
static const double ORACLE_PI = 3.141592653589793238462643383279502884;
static const double ORACLE_SQRT2 = 1.414213562373095048801688724209698079;

typedef struct {
  int dim;
  int shape[3];
  double L[3];
  double mu;
  double nu;
} oracle_hooke;

static void make_hooke(oracle_hooke* h, int dim, const int* shape,
                       const double* L, double mu, double nu) {
  h->dim = dim;
  for (int i = 0; i < 3; i++) {
    h->shape[i] = i < dim ? shape[i] : 1;
    h->L[i] = i < dim ? L[i] : 1.0;
  }
  h->mu = mu;
  h->nu = nu;
}

/* CartesianGrid::get_node_at, include/bri17/bri17.hpp:78-93. */
int oracle_get_node_at(int dim, const int* shape, const int* idx) {
  if (dim == 2) return idx[0] * shape[1] + idx[1];
  return (idx[0] * shape[1] + idx[1]) * shape[2] + idx[2];
}

/* CartesianGrid::get_cell_nodes, include/bri17/bri17.hpp:127-158.
 * Vertex order (i,j,k) -> {000,001,010,011,100,101,110,111}, periodic wrap. */
void oracle_get_cell_nodes(int dim, const int* shape, int cell, int* nodes) {
  if (dim == 2) {
    const int i1 = cell / shape[1];
    const int j1 = cell % shape[1];
    const int i2 = i1 == shape[0] - 1 ? 0 : i1 + 1;
    const int j2 = j1 == shape[1] - 1 ? 0 : j1 + 1;
    nodes[0] = i1 * shape[1] + j1;
    nodes[1] = i1 * shape[1] + j2;
    nodes[2] = i2 * shape[1] + j1;
    nodes[3] = i2 * shape[1] + j2;
  } else {
    const int k1 = cell % shape[2];
    const int ij1 = cell / shape[2];
    const int j1 = ij1 % shape[1];
    const int i1 = ij1 / shape[1];
    const int i2 = i1 == shape[0] - 1 ? 0 : i1 + 1;
    const int j2 = j1 == shape[1] - 1 ? 0 : j1 + 1;
    const int k2 = k1 == shape[2] - 1 ? 0 : k1 + 1;
#define NODE(i, j, k) (((i) * shape[1] + (j)) * shape[2] + (k))
    nodes[0] = NODE(i1, j1, k1);
    nodes[1] = NODE(i1, j1, k2);
    nodes[2] = NODE(i1, j2, k1);
    nodes[3] = NODE(i1, j2, k2);
    nodes[4] = NODE(i2, j1, k1);
    nodes[5] = NODE(i2, j1, k2);
    nodes[6] = NODE(i2, j2, k1);
    nodes[7] = NODE(i2, j2, k2);
#undef NODE
  }
}

/* Hooke::modal_strain_displacement, include/bri17/bri17.hpp:212-236.
 * B is DIM complex values. */
static void modal_strain_displacement(const oracle_hooke* h, const int* k,
                                      double* B) {
  double c[3], s[3];
  double sum_alpha = 0.0;
  for (int i = 0; i < h->dim; i++) {
    double alpha = ORACLE_PI * k[i] / h->shape[i];
    sum_alpha += alpha;
    c[i] = cos(alpha);
    s[i] = sin(alpha) * h->shape[i] / h->L[i];
  }
  const double pre_re = -2 * sin(sum_alpha);
  const double pre_im = 2 * cos(sum_alpha);
  /* std::complex<double> * double multiplies both parts, left to right. */
  if (h->dim == 2) {
    B[0] = pre_re * s[0] * c[1];
    B[1] = pre_im * s[0] * c[1];
    B[2] = pre_re * c[0] * s[1];
    B[3] = pre_im * c[0] * s[1];
  } else {
    B[0] = pre_re * s[0] * c[1] * c[2];
    B[1] = pre_im * s[0] * c[1] * c[2];
    B[2] = pre_re * c[0] * s[1] * c[2];
    B[3] = pre_im * c[0] * s[1] * c[2];
    B[4] = pre_re * c[0] * c[1] * s[2];
    B[5] = pre_im * c[0] * c[1] * s[2];
  }
}

/* Hooke::modal_stiffness, include/bri17/bri17.hpp:247-292.
 * Kr receives the DIM x DIM real parts (the imaginary parts are exactly 0
 * in the reference: every entry is built from real numbers). */
static void modal_stiffness_real(const oracle_hooke* h, const int* k,
                                 double* Kr) {
  double phi[3], psi[3], chi[3];
  for (int i = 0; i < h->dim; i++) {
    double hh = h->L[i] / h->shape[i];
    double beta = 2 * ORACLE_PI * k[i] / h->shape[i];
    phi[i] = 2 * (1 - cos(beta)) / hh / hh;
    chi[i] = (2 + cos(beta)) / 3;
    psi[i] = sin(beta) / hh;
  }
  const double scaling = h->mu / (1. - 2. * h->nu);
  if (h->dim == 2) {
    double H_00 = phi[0] * chi[1];
    double H_11 = chi[0] * phi[1];
    double K_diag = h->mu * (H_00 + H_11);
    Kr[0] = scaling * H_00 + K_diag;
    Kr[1] = scaling * psi[0] * psi[1];
    Kr[2] = Kr[1];
    Kr[3] = scaling * H_11 + K_diag;
  } else {
    double H_00 = phi[0] * chi[1] * chi[2];
    double H_11 = chi[0] * phi[1] * chi[2];
    double H_22 = chi[0] * chi[1] * phi[2];
    double K_diag = h->mu * (H_00 + H_11 + H_22);
    Kr[0] = scaling * H_00 + K_diag;
    Kr[1] = scaling * psi[0] * psi[1] * chi[2];
    Kr[2] = scaling * psi[0] * chi[1] * psi[2];
    Kr[3] = Kr[1];
    Kr[4] = scaling * H_11 + K_diag;
    Kr[5] = scaling * chi[0] * psi[1] * psi[2];
    Kr[6] = Kr[2];
    Kr[7] = Kr[5];
    Kr[8] = scaling * H_22 + K_diag;
  }
}

void oracle_modal_stiffness(int dim, const int* shape, const double* L,
                            double mu, double nu, const int* k, double* K) {
  oracle_hooke h;
  double Kr[9];
  make_hooke(&h, dim, shape, L, mu, nu);
  modal_stiffness_real(&h, k, Kr);
  for (int i = 0; i < dim * dim; i++) {
    K[2 * i] = Kr[i];
    K[2 * i + 1] = 0.0;
  }
}

void oracle_modal_strain_displacement(int dim, const int* shape,
                                      const double* L, double mu, double nu,
                                      const int* k, double* B) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  modal_strain_displacement(&h, k, B);
}

/* Batched forms over n multi-indices (k is n x dim, row-major). */
void oracle_modal_stiffness_batch(int dim, const int* shape, const double* L,
                                  double mu, double nu, const int* k,
                                  int64_t n, double* K) {
  for (int64_t m = 0; m < n; m++)
    oracle_modal_stiffness(dim, shape, L, mu, nu, k + m * dim,
                           K + m * 2 * dim * dim);
}

void oracle_modal_strain_displacement_batch(int dim, const int* shape,
                                            const double* L, double mu,
                                            double nu, const int* k, int64_t n,
                                            double* B) {
  for (int64_t m = 0; m < n; m++)
    oracle_modal_strain_displacement(dim, shape, L, mu, nu, k + m * dim,
                                     B + m * 2 * dim);
}

/* Hooke::modal_eigenstress_to_opposite_strain,
 * include/bri17/bri17.hpp:308-355.
 *
 * tau: sym complex values in Mandel order ((xx,yy,xy) in 2D,
 * (xx,yy,zz,yz,zx,xy) in 3D, sqrt(2) on the shears, :324-332).
 * The reference solves K u = tau . conj(B) with Eigen's LLT (:340-341); K is
 * real symmetric positive definite for k != 0, so this restatement factors it
 * with a real Cholesky and solves the real and imaginary parts.  k == 0
 * returns zeros (:336-339).  u_out (optional, DIM complex) receives the modal
 * solution u; eta receives sym(B (x) u) in Mandel form (:342-354). */
static void eigenstress_solve(const oracle_hooke* h, const int* k,
                              const double* tau, double* u_out, double* eta) {
  const int dim = h->dim;
  const int sym = dim == 2 ? 3 : 6;
  double B[6], Kr[9];
  modal_strain_displacement(h, k, B);
  modal_stiffness_real(h, k, Kr);
  int null_frequency = 1;
  for (int i = 0; i < dim; i++) null_frequency &= (k[i] == 0);
  if (null_frequency) {
    for (int i = 0; i < 2 * sym; i++) eta[i] = 0.0;
    if (u_out)
      for (int i = 0; i < 2 * dim; i++) u_out[i] = 0.0;
    return;
  }
  /* tau_mat (complex, symmetric) from Mandel components. */
  double tr[3][3], ti[3][3];
  if (dim == 2) {
    tr[0][0] = tau[0]; ti[0][0] = tau[1];
    tr[1][1] = tau[2]; ti[1][1] = tau[3];
    tr[0][1] = tr[1][0] = tau[4] / ORACLE_SQRT2;
    ti[0][1] = ti[1][0] = tau[5] / ORACLE_SQRT2;
  } else {
    tr[0][0] = tau[0]; ti[0][0] = tau[1];
    tr[1][1] = tau[2]; ti[1][1] = tau[3];
    tr[2][2] = tau[4]; ti[2][2] = tau[5];
    tr[1][2] = tr[2][1] = tau[6] / ORACLE_SQRT2;
    ti[1][2] = ti[2][1] = tau[7] / ORACLE_SQRT2;
    tr[0][2] = tr[2][0] = tau[8] / ORACLE_SQRT2;
    ti[0][2] = ti[2][0] = tau[9] / ORACLE_SQRT2;
    tr[0][1] = tr[1][0] = tau[10] / ORACLE_SQRT2;
    ti[0][1] = ti[1][0] = tau[11] / ORACLE_SQRT2;
  }
  /* rhs = tau_mat * conj(B). */
  double rr[3], ri[3];
  for (int i = 0; i < dim; i++) {
    double sr = 0.0, si = 0.0;
    for (int j = 0; j < dim; j++) {
      const double br = B[2 * j], bi = -B[2 * j + 1];
      sr += tr[i][j] * br - ti[i][j] * bi;
      si += tr[i][j] * bi + ti[i][j] * br;
    }
    rr[i] = sr;
    ri[i] = si;
  }
  /* Cholesky K = L L^T (K row-major in Kr), then two triangular solves. */
  double Lc[3][3] = {{0}};
  for (int j = 0; j < dim; j++) {
    double d = Kr[j * dim + j];
    for (int p = 0; p < j; p++) d -= Lc[j][p] * Lc[j][p];
    d = sqrt(d);
    Lc[j][j] = d;
    for (int i = j + 1; i < dim; i++) {
      double s = Kr[i * dim + j];
      for (int p = 0; p < j; p++) s -= Lc[i][p] * Lc[j][p];
      Lc[i][j] = s / d;
    }
  }
  double yr[3], yi[3], ur[3], ui[3];
  for (int i = 0; i < dim; i++) {
    double sr = rr[i], si = ri[i];
    for (int p = 0; p < i; p++) {
      sr -= Lc[i][p] * yr[p];
      si -= Lc[i][p] * yi[p];
    }
    yr[i] = sr / Lc[i][i];
    yi[i] = si / Lc[i][i];
  }
  for (int i = dim - 1; i >= 0; i--) {
    double sr = yr[i], si = yi[i];
    for (int p = i + 1; p < dim; p++) {
      sr -= Lc[p][i] * ur[p];
      si -= Lc[p][i] * ui[p];
    }
    ur[i] = sr / Lc[i][i];
    ui[i] = si / Lc[i][i];
  }
  if (u_out)
    for (int i = 0; i < dim; i++) {
      u_out[2 * i] = ur[i];
      u_out[2 * i + 1] = ui[i];
    }
  /* eta_mat = 0.5 * (B u^T + u B^T) (no conjugation, :342). */
#define EPS_RE(i, j) \
  (0.5 * ((B[2 * (i)] * ur[j] - B[2 * (i) + 1] * ui[j]) + \
          (ur[i] * B[2 * (j)] - ui[i] * B[2 * (j) + 1])))
#define EPS_IM(i, j) \
  (0.5 * ((B[2 * (i)] * ui[j] + B[2 * (i) + 1] * ur[j]) + \
          (ur[i] * B[2 * (j) + 1] + ui[i] * B[2 * (j)])))
  if (dim == 2) {
    eta[0] = EPS_RE(0, 0); eta[1] = EPS_IM(0, 0);
    eta[2] = EPS_RE(1, 1); eta[3] = EPS_IM(1, 1);
    eta[4] = ORACLE_SQRT2 * EPS_RE(0, 1); eta[5] = ORACLE_SQRT2 * EPS_IM(0, 1);
  } else {
    eta[0] = EPS_RE(0, 0); eta[1] = EPS_IM(0, 0);
    eta[2] = EPS_RE(1, 1); eta[3] = EPS_IM(1, 1);
    eta[4] = EPS_RE(2, 2); eta[5] = EPS_IM(2, 2);
    eta[6] = ORACLE_SQRT2 * EPS_RE(1, 2); eta[7] = ORACLE_SQRT2 * EPS_IM(1, 2);
    eta[8] = ORACLE_SQRT2 * EPS_RE(2, 0); eta[9] = ORACLE_SQRT2 * EPS_IM(2, 0);
    eta[10] = ORACLE_SQRT2 * EPS_RE(0, 1); eta[11] = ORACLE_SQRT2 * EPS_IM(0, 1);
  }
#undef EPS_RE
#undef EPS_IM
}

void oracle_modal_eigenstress_to_opposite_strain(int dim, const int* shape,
                                                 const double* L, double mu,
                                                 double nu, const int* k,
                                                 const double* tau,
                                                 double* eta) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  eigenstress_solve(&h, k, tau, 0, eta);
}

/* Row-major multi-index of flat position m over the full frequency grid,
 * the order of the nested k loops at tests/test_bri17.cpp:63-91. */
static void unflatten(const oracle_hooke* h, int64_t m, int* k) {
  for (int i = h->dim - 1; i >= 0; i--) {
    k[i] = (int)(m % h->shape[i]);
    m /= h->shape[i];
  }
}

/* The per-mode loop of StiffnessMatrixFactory::compute_Ku,
 * tests/test_bri17.cpp:58-92: Ku_hat[k] = K(k) u_hat[k] for every k of the
 * full spectrum.  uhat and Kuhat are DIM x size complex (SoA). */
void oracle_stiffness_modal_apply(int dim, const int* shape, const double* L,
                                  double mu, double nu, const double* uhat,
                                  double* Kuhat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= shape[i];
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double Kr[9];
    unflatten(&h, m, k);
    modal_stiffness_real(&h, k, Kr);
    for (int r = 0; r < dim; r++) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j < dim; j++) {
        sr += Kr[r * dim + j] * uhat[2 * (j * size + m)];
        si += Kr[r * dim + j] * uhat[2 * (j * size + m) + 1];
      }
      Kuhat[2 * (r * size + m)] = sr;
      Kuhat[2 * (r * size + m) + 1] = si;
    }
  }
}

/* The per-mode loop of StrainDisplacementMatrixFactory::compute_Bu,
 * tests/test_bri17.cpp:196-235: eps_hat[k] = sym(B(k) (x) u_hat[k]) with
 * sqrt(2) on the shears.  Output is sym x size complex (SoA). */
void oracle_strain_modal_apply(int dim, const int* shape, const double* L,
                               double mu, double nu, const double* uhat,
                               double* epshat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= shape[i];
  static const int pairs2[3][2] = {{0, 0}, {1, 1}, {0, 1}};
  static const int pairs3[6][2] = {{0, 0}, {1, 1}, {2, 2},
                                   {1, 2}, {2, 0}, {0, 1}};
  const int sym = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double B[6], ur[3], ui[3];
    unflatten(&h, m, k);
    modal_strain_displacement(&h, k, B);
    for (int j = 0; j < dim; j++) {
      ur[j] = uhat[2 * (j * size + m)];
      ui[j] = uhat[2 * (j * size + m) + 1];
    }
    for (int s = 0; s < sym; s++) {
      const int i = dim == 2 ? pairs2[s][0] : pairs3[s][0];
      const int j = dim == 2 ? pairs2[s][1] : pairs3[s][1];
      double er = 0.5 * ((B[2 * i] * ur[j] - B[2 * i + 1] * ui[j]) +
                         (ur[i] * B[2 * j] - ui[i] * B[2 * j + 1]));
      double ei = 0.5 * ((B[2 * i] * ui[j] + B[2 * i + 1] * ur[j]) +
                         (ur[i] * B[2 * j + 1] + ui[i] * B[2 * j]));
      if (i != j) {
        er *= ORACLE_SQRT2;
        ei *= ORACLE_SQRT2;
      }
      epshat[2 * (s * size + m)] = er;
      epshat[2 * (s * size + m) + 1] = ei;
    }
  }
}

/* Modal direct solve of the eigenstress problem over the full spectrum:
 * u_hat[k] solves K(k) u_hat[k] = tau_hat[k] . conj(B(k)) (the linear system
 * of include/bri17/bri17.hpp:340-341), u_hat[0] = 0.  tauhat is sym x size
 * complex (SoA, Mandel); uhat is DIM x size complex (SoA).  The solution of
 * the real-space problem K u = -|h| B^T tau is then -ifft(u_hat), the sign
 * convention of the reference's "opposite strain". */
void oracle_eigenstress_modal_solve(int dim, const int* shape, const double* L,
                                    double mu, double nu, const double* tauhat,
                                    double* uhat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= shape[i];
  const int sym = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double tau[12], u[6], eta[12];
    unflatten(&h, m, k);
    for (int s = 0; s < sym; s++) {
      tau[2 * s] = tauhat[2 * (s * size + m)];
      tau[2 * s + 1] = tauhat[2 * (s * size + m) + 1];
    }
    eigenstress_solve(&h, k, tau, u, eta);
    for (int j = 0; j < dim; j++) {
      uhat[2 * (j * size + m)] = u[2 * j];
      uhat[2 * (j * size + m) + 1] = u[2 * j + 1];
    }
  }
}

/* The same modal direct solve over the half spectrum of a real field: the
 * last axis holds only k_last in [0, shape[dim-1]/2] (the layout of a
 * real-to-complex DFT), every other axis its full range.  tauhat is
 * sym x (size / shape[dim-1] * H) complex (SoA) with H = shape[dim-1]/2 + 1,
 * uhat DIM x that.  Every mode k is solved exactly as by
 * oracle_eigenstress_modal_solve; the modes left out are the complex
 * conjugates of kept ones (K(-k) = K(k), B(-k) = conj(B(k))), which the
 * inverse real DFT restores. */
void oracle_eigenstress_modal_solve_half(int dim, const int* shape, const double* L,
                                         double mu, double nu, const double* tauhat,
                                         double* uhat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  oracle_hooke hh = h;
  hh.shape[dim - 1] = shape[dim - 1] / 2 + 1;
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= hh.shape[i];
  const int sym = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double tau[12], u[6], eta[12];
    unflatten(&hh, m, k);
    for (int s = 0; s < sym; s++) {
      tau[2 * s] = tauhat[2 * (s * size + m)];
      tau[2 * s + 1] = tauhat[2 * (s * size + m) + 1];
    }
    eigenstress_solve(&h, k, tau, u, eta);
    for (int j = 0; j < dim; j++) {
      uhat[2 * (j * size + m)] = u[2 * j];
      uhat[2 * (j * size + m) + 1] = u[2 * j + 1];
    }
  }
}

/* Opposite strain in Fourier space over the full spectrum: eta_hat[k] =
 * Hooke::modal_eigenstress_to_opposite_strain(k, tau_hat[k])
 * (include/bri17/bri17.hpp:308-355), the per-mode loop of
 * python/demo.py:34-40.  tauhat and etahat are sym x size complex (SoA). */
void oracle_eigenstress_modal_eta(int dim, const int* shape, const double* L, double mu,
                                  double nu, const double* tauhat, double* etahat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= shape[i];
  const int sym = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double tau[12], eta[12];
    unflatten(&h, m, k);
    for (int s = 0; s < sym; s++) {
      tau[2 * s] = tauhat[2 * (s * size + m)];
      tau[2 * s + 1] = tauhat[2 * (s * size + m) + 1];
    }
    eigenstress_solve(&h, k, tau, 0, eta);
    for (int s = 0; s < sym; s++) {
      etahat[2 * (s * size + m)] = eta[2 * s];
      etahat[2 * (s * size + m) + 1] = eta[2 * s + 1];
    }
  }
}

/* Eigenstress right-hand side in Fourier space: b_hat[k] = tau_hat[k] .
 * conj(B(k)) (the rhs of include/bri17/bri17.hpp:340), DIM x size complex. */
void oracle_eigenstress_modal_rhs(int dim, const int* shape, const double* L,
                                  double mu, double nu, const double* tauhat,
                                  double* bhat) {
  oracle_hooke h;
  make_hooke(&h, dim, shape, L, mu, nu);
  int64_t size = 1;
  for (int i = 0; i < dim; i++) size *= shape[i];
  static const int pairs2[3][2] = {{0, 0}, {1, 1}, {0, 1}};
  static const int pairs3[6][2] = {{0, 0}, {1, 1}, {2, 2},
                                   {1, 2}, {2, 0}, {0, 1}};
  const int sym = dim == 2 ? 3 : 6;
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < size; m++) {
    int k[3];
    double B[6];
    double tr[3][3] = {{0}}, ti[3][3] = {{0}};
    unflatten(&h, m, k);
    modal_strain_displacement(&h, k, B);
    for (int s = 0; s < sym; s++) {
      const int i = dim == 2 ? pairs2[s][0] : pairs3[s][0];
      const int j = dim == 2 ? pairs2[s][1] : pairs3[s][1];
      double vr = tauhat[2 * (s * size + m)];
      double vi = tauhat[2 * (s * size + m) + 1];
      if (i != j) {
        vr /= ORACLE_SQRT2;
        vi /= ORACLE_SQRT2;
      }
      tr[i][j] = tr[j][i] = vr;
      ti[i][j] = ti[j][i] = vi;
    }
    for (int i = 0; i < dim; i++) {
      double sr = 0.0, si = 0.0;
      for (int j = 0; j < dim; j++) {
        const double br = B[2 * j], bi = -B[2 * j + 1];
        sr += tr[i][j] * br - ti[i][j] * bi;
        si += tr[i][j] * bi + ti[i][j] * br;
      }
      bhat[2 * (i * size + m)] = sr;
      bhat[2 * (i * size + m) + 1] = si;
    }
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
