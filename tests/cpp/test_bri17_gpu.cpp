// C++ counterpart of the reference's TEST_CASE("Global assembly tests")
// (tests/test_bri17.cpp:318-606), written against this library's C++ host
// API (include/bri17/bri17_gpu.hpp): for each section the dense global K
// (or B) is extracted from the GPU operator by unit vectors, as
// StiffnessMatrixFactory::run / StrainDisplacementMatrixFactory::run do
// (:130-150, :271-292), and compared with the real-space assembly of the
// Maxima element matrix (:153-174, :295-316) with |a - e| <= rtol |e| + atol.
//
// Usage: test_bri17_gpu <golden.txt>, one case per line:
//   <K|B> <dim> <shape...> <L...> <mu> <nu> <rtol> <atol> <rows> <cols> <values...>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bri17/bri17_gpu.hpp"

namespace {

template <int DIM>
std::vector<double> assemble(const bri17::CartesianGrid<double, DIM>& grid,
                             const std::vector<double>& Ee, int rows, int cols, bool stiffness) {
  const int nn = grid.num_nodes_per_cell;
  const int sym = DIM == 2 ? 3 : 6;
  const int ndof = DIM * grid.size;
  const int nrow = stiffness ? ndof : sym * grid.size;
  std::vector<double> M((size_t)nrow * ndof, 0.0);
  for (int cell = 0; cell < grid.size; cell++) {
    auto nodes = grid.get_cell_nodes(cell);
    for (int ie = 0; ie < rows; ie++) {
      const int i = stiffness ? nodes[ie % nn] + grid.size * (ie / nn) : ie * grid.size + cell;
      for (int je = 0; je < cols; je++) {
        const int j = nodes[je % nn] + grid.size * (je / nn);
        M[(size_t)i * ndof + j] += Ee[(size_t)ie * cols + je];
      }
    }
  }
  return M;
}

template <int DIM>
std::vector<double> extract(const bri17::Hooke<double, DIM>& h, bool stiffness, int* nrow_out) {
  const int sym = DIM == 2 ? 3 : 6;
  const int ndof = DIM * h.grid.size;
  const int nrow = stiffness ? ndof : sym * h.grid.size;
  *nrow_out = nrow;
  double *u = nullptr, *f = nullptr;
  cudaMalloc(&u, sizeof(double) * ndof);
  cudaMalloc(&f, sizeof(double) * nrow);
  std::vector<double> M((size_t)nrow * ndof), col(nrow);
  const double one = 1.0;
  for (int j = 0; j < ndof; j++) {
    cudaMemset(u, 0, sizeof(double) * ndof);
    cudaMemcpy(u + j, &one, sizeof(double), cudaMemcpyHostToDevice);
    if (stiffness)
      h.apply_stiffness(u, f);
    else
      h.apply_strain(u, f);
    cudaMemcpy(col.data(), f, sizeof(double) * nrow, cudaMemcpyDeviceToHost);
    for (int i = 0; i < nrow; i++) M[(size_t)i * ndof + j] = col[i];
  }
  cudaFree(u);
  cudaFree(f);
  return M;
}

template <int DIM>
bool run_case(std::istringstream& in, const std::string& kind) {
  std::array<int, DIM> shape;
  std::array<double, DIM> L;
  for (auto& n : shape) in >> n;
  for (auto& x : L) in >> x;
  double mu, nu, rtol, atol;
  int rows, cols;
  in >> mu >> nu >> rtol >> atol >> rows >> cols;
  std::vector<double> Ee((size_t)rows * cols);
  for (auto& v : Ee) in >> v;
  bri17::CartesianGrid<double, DIM> grid{shape, L};
  bri17::Hooke<double, DIM> hooke{mu, nu, grid};
  const bool stiffness = kind == "K";
  int nrow = 0;
  auto actual = extract<DIM>(hooke, stiffness, &nrow);
  auto expected = assemble<DIM>(grid, Ee, rows, cols, stiffness);
  int bad = 0;
  for (size_t i = 0; i < expected.size(); i++) {
    const double tol = rtol * std::fabs(expected[i]) + atol;
    if (!(std::fabs(actual[i] - expected[i]) <= tol)) {
      if (bad < 5)
        std::printf("  [%zu, %zu]: expected = %.17g, actual = %.17g\n", i / (DIM * grid.size),
                    i % (DIM * grid.size), expected[i], actual[i]);
      bad++;
    }
  }
  std::printf("%dD %s matrix (%s): %s (%d mismatches of %zu)\n", DIM,
              stiffness ? "stiffness" : "strain-displacement", hooke.repr().c_str(),
              bad ? "FAILED" : "passed", bad, expected.size());
  return bad == 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s golden.txt\n", argv[0]);
    return 2;
  }
  std::ifstream f(argv[1]);
  std::string line;
  int passed = 0, total = 0;
  try {
    while (std::getline(f, line)) {
      if (line.empty()) continue;
      std::istringstream in(line);
      std::string kind;
      int dim;
      in >> kind >> dim;
      const bool ok = dim == 2 ? run_case<2>(in, kind) : run_case<3>(in, kind);
      passed += ok;
      total++;
    }
  } catch (const std::exception& e) {
    std::printf("exception: %s\n", e.what());
    return 1;
  }
  // T = float instantiation of the header API (`scaling` promoted to double,
  // include/bri17/bri17.hpp:266): the FP32 operator
  // agrees with the FP64 one to FP32 accuracy, and the per-mode methods
  // return the FP64 values rounded to float.
  {
    bri17::CartesianGrid<float, 3> g32{{8, 6, 10}, {1.f, 0.75f, 1.25f}};
    bri17::CartesianGrid<double, 3> g64{{8, 6, 10}, {1.0, 0.75, 1.25}};
    bri17::Hooke<float, 3> h32{1.5f, 0.25f, g32};  // nu exact in float and double
    bri17::Hooke<double, 3> h64{1.5, 0.25, g64};
    const int n = 3 * g64.size;
    std::vector<double> u64(n), f64(n), f32d(n);
    std::vector<float> u32(n), f32(n);
    unsigned s = 12345u;
    for (int i = 0; i < n; i++) {
      s = s * 1103515245u + 12345u;
      u32[i] = (float)((s >> 8) % 2001) / 1000.f - 1.f;
      u64[i] = u32[i];
    }
    h64.apply_stiffness_host(u64.data(), f64.data());
    h32.apply_stiffness_host(u32.data(), f32.data());
    double num = 0, den = 0;
    for (int i = 0; i < n; i++) {
      num += (f32[i] - f64[i]) * (f32[i] - f64[i]);
      den += f64[i] * f64[i];
    }
    const double rel = std::sqrt(num / den);
    int k[3] = {3, 2, 7};
    std::complex<float> K32[9];
    std::complex<double> K64[9];
    h32.modal_stiffness(k, K32);
    h64.modal_stiffness(k, K64);
    bool modal_ok = true;
    for (int i = 0; i < 9; i++)
      modal_ok = modal_ok && K32[i] == std::complex<float>(K64[i]);
    const bool ok = rel <= 2e-5 && modal_ok;
    std::printf("Hooke<float,3>: operator rel err %.2e vs FP64, modal %s: %s\n", rel,
                modal_ok ? "equal" : "differ", ok ? "passed" : "FAILED");
    passed += ok;
    total++;
  }
  // Float-pair arithmetic on an FP64 handle (Hooke<double,3>::set_float_pair):
  // within 1e-13 of the FP64 operator, and switching back gives the FP64
  // result bit for bit.
  {
    bri17::CartesianGrid<double, 3> g{{64, 64, 128}, {1.0, 1.0, 2.0}};
    bri17::Hooke<double, 3> h{1.0, 0.3, g};
    const int n = 3 * g.size;
    std::vector<double> u(n), f(n), fp(n), f2(n);
    unsigned s = 777u;
    for (int i = 0; i < n; i++) {
      s = s * 1103515245u + 12345u;
      u[i] = (double)((s >> 8) % 20001) / 10000.0 - 1.0;
    }
    h.apply_stiffness_host(u.data(), f.data());
    h.set_float_pair(true);
    h.apply_stiffness_host(u.data(), fp.data());
    h.set_float_pair(false);
    h.apply_stiffness_host(u.data(), f2.data());
    double num = 0, den = 0;
    bool same = true;
    for (int i = 0; i < n; i++) {
      num += (fp[i] - f[i]) * (fp[i] - f[i]);
      den += f[i] * f[i];
      same = same && f2[i] == f[i];
    }
    const double rel = std::sqrt(num / den);
    const bool ok = rel <= 1e-13 && same;
    std::printf("Hooke<double,3> float pairs: rel diff %.2e vs FP64, FP64 again %s: %s\n", rel,
                same ? "identical" : "differs", ok ? "passed" : "FAILED");
    passed += ok;
    total++;
  }
  std::printf("%d of %d sections passed\n", passed, total);
  return passed == total && total > 0 ? 0 : 1;
}
