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
  std::printf("%d of %d sections passed\n", passed, total);
  return passed == total && total > 0 ? 0 : 1;
}
