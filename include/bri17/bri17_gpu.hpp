/**
 * bri17_gpu.hpp -- C++ host API of the GB300 library, mirroring the
 * reference's header-only API (include/bri17/bri17.hpp of sbrisard/bri17):
 * class templates bri17::CartesianGrid<T,DIM> and bri17::Hooke<T,DIM> with
 * the same members, constructors and per-mode signatures, plus whole-field
 * methods.  Every numerical method runs on the GPU through the C ABI of
 * bri17_gb300.h; per-mode calls are batches of one.
 *
 * Errors: std::invalid_argument for invalid arguments, std::runtime_error for
 * every other failure status (the reference throws only from unreachable
 * branches, include/bri17/bri17.hpp:154-156).
 */
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <complex>
#include <cstdint>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <typeinfo>

#include "../bri17_gb300.h"

namespace bri17 {

namespace detail {
inline void check(int status, const char* where) {
  if (status == BRI17_OK) return;
  std::string msg = std::string(where) + ": " + bri17_status_string(status);
  const char* d = bri17_last_error();
  if (d && *d) msg += std::string(" (") + d + ")";
  if (status == BRI17_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

}  // namespace detail

/** A rectangular periodic grid (include/bri17/bri17.hpp:34-159). */
template <typename T, int DIM>
class CartesianGrid {
  static_assert(std::is_floating_point<T>::value && (DIM == 2 || DIM == 3),
                "CartesianGrid<T, DIM>: T floating point, DIM 2 or 3");

 public:
  static constexpr int num_nodes_per_cell = 1 << DIM;
  std::array<int, DIM> const shape;
  std::array<T, DIM> const L;
  int const size;

  CartesianGrid(std::array<int, DIM> shape, std::array<T, DIM> L)
      : shape{shape}, L{L}, size{product(shape)} {}

  std::string repr() const {
    std::ostringstream s;
    s << "CartesianGrid<" << typeid(T).name() << "," << DIM << ">{shape={";
    for (auto n : shape) s << n << ",";
    s << "},L={";
    for (auto x : L) s << x << ",";
    s << "}}";
    return s.str();
  }

  int get_node_at(int i, int j) const {
    static_assert(DIM == 2, "this method expects a 2D grid");
    return i * shape[1] + j;
  }
  int get_node_at(int i, int j, int k) const {
    static_assert(DIM == 3, "this method expects a 3D grid");
    return (i * shape[1] + j) * shape[2] + k;
  }

  /** Periodic vertices of a cell; vertex v has axis-d offset bit
   *  (v >> (DIM-1-d)) & 1, the order of include/bri17/bri17.hpp:127-158. */
  std::array<int, num_nodes_per_cell> get_cell_nodes(int cell) const {
    int idx[DIM], nxt[DIM];
    for (int d = DIM - 1; d >= 0; d--) {
      idx[d] = cell % shape[d];
      cell /= shape[d];
      nxt[d] = idx[d] == shape[d] - 1 ? 0 : idx[d] + 1;
    }
    std::array<int, num_nodes_per_cell> nodes;
    for (int v = 0; v < num_nodes_per_cell; v++) {
      int n = 0;
      for (int d = 0; d < DIM; d++)
        n = n * shape[d] + (((v >> (DIM - 1 - d)) & 1) ? nxt[d] : idx[d]);
      nodes[v] = n;
    }
    return nodes;
  }

 private:
  static int product(const std::array<int, DIM>& s) {
    int p = 1;
    for (int n : s) p *= n;
    return p;
  }
};

template <typename T, int DIM>
std::ostream& operator<<(std::ostream& os, const CartesianGrid<T, DIM>& g) {
  return os << g.repr();
}

/** Isotropic Hooke material on a periodic grid, with its GPU operator
 *  (include/bri17/bri17.hpp:176-356). */
template <typename T, int DIM>
class Hooke {
  static_assert((std::is_same<T, float>::value || std::is_same<T, double>::value) &&
                    (DIM == 2 || DIM == 3),
                "Hooke<T, DIM>: T float or double (the operator's field types), DIM 2 or 3");

 public:
  T const mu;
  T const nu;
  CartesianGrid<T, DIM> const grid;
  static constexpr int sym = DIM == 2 ? 3 : 6;

  Hooke(T mu, T nu, CartesianGrid<T, DIM>& grid) : mu{mu}, nu{nu}, grid{grid} { create(); }
  Hooke(const Hooke& o) : mu{o.mu}, nu{o.nu}, grid{o.grid} { create(); }
  Hooke& operator=(const Hooke&) = delete;
  ~Hooke() { bri17_op_destroy(op_); }

  std::string repr() const {
    std::ostringstream s;
    s << "Hooke<" << typeid(T).name() << "," << DIM << ">{mu=" << mu << ",nu=" << nu
      << ",grid=" << grid << std::endl;
    return s.str();
  }

  /** Hooke::modal_strain_displacement (:212-236): B has DIM entries.  One
   *  kernel on the GPU per call (page-locked staging kept by the handle, no
   *  allocation per call); batches amortise the launch. */
  void modal_strain_displacement(int const* k, std::complex<T>* B) const {
    std::complex<double> out[DIM];
    detail::check(bri17_modal_strain_displacement_host(op_, k, 1, out),
                  "bri17_modal_strain_displacement_host");
    for (int i = 0; i < DIM; i++) B[i] = std::complex<T>(out[i]);
  }

  /** Hooke::modal_stiffness (:247-292): K has DIM*DIM entries (row-major). */
  void modal_stiffness(int const* k, std::complex<T>* K) const {
    std::complex<double> out[DIM * DIM];
    detail::check(bri17_modal_stiffness_host(op_, k, 1, out), "bri17_modal_stiffness_host");
    for (int i = 0; i < DIM * DIM; i++) K[i] = std::complex<T>(out[i]);
  }

  /** Hooke::modal_eigenstress_to_opposite_strain (:308-355). */
  void modal_eigenstress_to_opposite_strain(int const* k, std::complex<T> const* tau,
                                            std::complex<T>* eta) const {
    std::complex<double> t[sym], e[sym];
    for (int i = 0; i < sym; i++) t[i] = std::complex<double>(tau[i]);
    detail::check(bri17_modal_eigenstress_to_opposite_strain_host(op_, k, 1, t, e),
                  "bri17_modal_eigenstress_to_opposite_strain_host");
    for (int i = 0; i < sym; i++) eta[i] = std::complex<T>(e[i]);
  }

  /** Batched per-mode functions on host buffers (n modes; k is n x DIM,
   *  outputs n x DIM*DIM / n x DIM complex, in double as the reference's
   *  per-mode arithmetic runs in double). */
  void modal_stiffness_batch(int const* k, int64_t n, std::complex<double>* K) const {
    detail::check(bri17_modal_stiffness_host(op_, k, n, K), "bri17_modal_stiffness_host");
  }
  void modal_strain_displacement_batch(int const* k, int64_t n,
                                       std::complex<double>* B) const {
    detail::check(bri17_modal_strain_displacement_host(op_, k, n, B),
                  "bri17_modal_strain_displacement_host");
  }

  // -- whole-field methods on device buffers (SoA, row-major nodes) ------
  /** f = K u, StiffnessMatrixFactory::compute_Ku (tests/test_bri17.cpp:56-107). */
  void apply_stiffness(T const* u_dev, T* f_dev, cudaStream_t s = nullptr) const {
    detail::check(bri17_apply_stiffness(op_, u_dev, f_dev, s), "bri17_apply_stiffness");
  }
  /** Same with host buffers (synchronous; page-locked buffers are read and
   *  written in place by the first and last passes). */
  void apply_stiffness_host(T const* u, T* f, cudaStream_t s = nullptr) const {
    detail::check(bri17_apply_stiffness_host(op_, u, f, s), "bri17_apply_stiffness_host");
  }
  /** T = double: apply_stiffness(_host) in float-pair arithmetic on the FP32
   *  pipe (about 1e-14 from FP64); 3D power-of-two grids only. */
  template <typename U = T,
            typename = typename std::enable_if<std::is_same<U, double>::value>::type>
  void set_float_pair(bool enable) {
    detail::check(bri17_op_set_float_pair(op_, enable ? 1 : 0), "bri17_op_set_float_pair");
  }
  /** Cell strains (Mandel), compute_Bu (tests/test_bri17.cpp:194-245). */
  void apply_strain(T const* u_dev, T* eps_dev, cudaStream_t s = nullptr) const {
    detail::check(bri17_apply_strain(op_, u_dev, eps_dev, s), "bri17_apply_strain");
  }
  /** Nodal forces b = -|h| B^T tau of a Mandel eigenstress. */
  void eigenstress_rhs(T const* tau_dev, T* b_dev, cudaStream_t s = nullptr) const {
    detail::check(bri17_eigenstress_rhs(op_, tau_dev, b_dev, s), "bri17_eigenstress_rhs");
  }
  /** Opposite strain field of a Mandel eigenstress field: the whole-field
   *  modal_eigenstress_to_opposite_strain (:308-355), sym x size. */
  void eigenstress_to_opposite_strain(T const* tau_dev, T* eta_dev,
                                      cudaStream_t s = nullptr) const {
    detail::check(bri17_eigenstress_to_opposite_strain(op_, tau_dev, eta_dev, s),
                  "bri17_eigenstress_to_opposite_strain");
  }
  /** CG solve of K x = b (FP64 vectors); mixed = FP32 inner + FP64 refinement. */
  bri17_cg_info cg_solve(double const* b_dev, double* x_dev, double tol, int max_iterations,
                         bool mixed = false, cudaStream_t s = nullptr) const {
    bri17_cg_info info;
    int rc = bri17_cg_solve(op_, b_dev, x_dev, tol, max_iterations,
                            mixed ? BRI17_CG_MIXED : BRI17_CG_PLAIN, &info, s);
    if (rc != BRI17_OK && rc != BRI17_ERR_NOT_CONVERGED) detail::check(rc, "bri17_cg_solve");
    return info;
  }

  bri17_op* handle() const { return op_; }

 private:
  bri17_op* op_ = nullptr;

  void create() {
    int shape[DIM];
    double L[DIM];
    for (int i = 0; i < DIM; i++) {
      shape[i] = grid.shape[i];
      L[i] = grid.L[i];
    }
    const int prec = std::is_same<T, float>::value ? BRI17_F32 : BRI17_F64;
    detail::check(bri17_op_create(DIM, shape, L, mu, nu, prec, &op_), "bri17_op_create");
  }

};

template <typename T, int DIM>
std::ostream& operator<<(std::ostream& os, const Hooke<T, DIM>& h) {
  return os << h.repr();
}

}  // namespace bri17
