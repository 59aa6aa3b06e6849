// ref_wrap.cpp -- C entry points over the UNMODIFIED reference header.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
// reference's include/bri17/bri17.hpp where it lies (never copied into this
// repository) into oracle/_ref/libbri17_ref.so.  Tests use it to pin the C
// restatement in oracle/bri17_oracle.c and to write the golden fixtures.
#include <array>
#include <complex>
#include <sstream>
#include <typeinfo>

#include "bri17/bri17.hpp"

namespace {
template <int DIM>
bri17::Hooke<double, DIM> make(const int* shape, const double* L, double mu,
                               double nu) {
  std::array<int, DIM> s;
  std::array<double, DIM> l;
  for (int i = 0; i < DIM; i++) {
    s[i] = shape[i];
    l[i] = L[i];
  }
  bri17::CartesianGrid<double, DIM> grid{s, l};
  return bri17::Hooke<double, DIM>{mu, nu, grid};
}
}  // namespace

extern "C" {

// Hooke<double,DIM>::modal_stiffness over n multi-indices (k: n x dim).
void ref_modal_stiffness_batch(int dim, const int* shape, const double* L,
                               double mu, double nu, const int* k, long n,
                               double* K) {
  auto* out = reinterpret_cast<std::complex<double>*>(K);
  if (dim == 2) {
    auto h = make<2>(shape, L, mu, nu);
    for (long m = 0; m < n; m++) h.modal_stiffness(k + 2 * m, out + 4 * m);
  } else {
    auto h = make<3>(shape, L, mu, nu);
    for (long m = 0; m < n; m++) h.modal_stiffness(k + 3 * m, out + 9 * m);
  }
}

// Hooke<double,DIM>::modal_strain_displacement over n multi-indices.
void ref_modal_strain_displacement_batch(int dim, const int* shape,
                                         const double* L, double mu, double nu,
                                         const int* k, long n, double* B) {
  auto* out = reinterpret_cast<std::complex<double>*>(B);
  if (dim == 2) {
    auto h = make<2>(shape, L, mu, nu);
    for (long m = 0; m < n; m++)
      h.modal_strain_displacement(k + 2 * m, out + 2 * m);
  } else {
    auto h = make<3>(shape, L, mu, nu);
    for (long m = 0; m < n; m++)
      h.modal_strain_displacement(k + 3 * m, out + 3 * m);
  }
}

// CartesianGrid<double,DIM>::get_cell_nodes for every cell (nodes: size x 2^dim).
void ref_all_cell_nodes(int dim, const int* shape, int* nodes) {
  if (dim == 2) {
    bri17::CartesianGrid<double, 2> g{{shape[0], shape[1]}, {1.0, 1.0}};
    for (int c = 0; c < g.size; c++) {
      auto v = g.get_cell_nodes(c);
      for (int i = 0; i < 4; i++) nodes[4 * c + i] = v[i];
    }
  } else {
    bri17::CartesianGrid<double, 3> g{{shape[0], shape[1], shape[2]},
                                      {1.0, 1.0, 1.0}};
    for (int c = 0; c < g.size; c++) {
      auto v = g.get_cell_nodes(c);
      for (int i = 0; i < 8; i++) nodes[8 * c + i] = v[i];
    }
  }
}

// CartesianGrid::repr and Hooke::repr (for the string-format parity test).
int ref_repr(int dim, const int* shape, const double* L, double mu, double nu,
             int which, char* buf, int cap) {
  std::string s;
  if (dim == 2) {
    auto h = make<2>(shape, L, mu, nu);
    s = which == 0 ? h.grid.repr() : h.repr();
  } else {
    auto h = make<3>(shape, L, mu, nu);
    s = which == 0 ? h.grid.repr() : h.repr();
  }
  int n = (int)s.size();
  if (n + 1 > cap) return -n;
  for (int i = 0; i < n; i++) buf[i] = s[i];
  buf[n] = 0;
  return n;
}
}
