"""CPU checks of the C ABI library: it loads without a GPU, exports every
function include/bri17_gb300.h declares, and validates its arguments before
touching a device."""
import ctypes

import numpy as np
import pytest

from bri17_gb300 import _lib
from conftest import gpu_available


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    declared = _lib.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_every_declared_symbol_has_a_python_signature():
    assert set(_lib.declared_symbols()) <= set(_lib._SIGS)


def test_status_strings_and_version():
    L = _lib.load()
    for code, text in _lib.STATUS.items():
        assert L.bri17_status_string(code).decode().startswith(text.split()[0])
    assert L.bri17_version().decode() == "0.1.0"


def test_argument_validation_before_device():
    L = _lib.load()
    h = ctypes.c_void_p()
    shape = (ctypes.c_int * 3)(8, 8, 8)
    Ls = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    assert L.bri17_op_create(4, shape, Ls, 1.0, 0.3, 0, ctypes.byref(h)) == 1
    assert L.bri17_op_create(3, shape, Ls, 1.0, 0.5, 0, ctypes.byref(h)) == 1
    assert L.bri17_op_create(3, shape, Ls, -1.0, 0.3, 0, ctypes.byref(h)) == 1
    assert L.bri17_op_create(3, shape, Ls, 1.0, 0.3, 7, ctypes.byref(h)) == 1
    bad = (ctypes.c_int * 3)(8, 0, 8)
    assert L.bri17_op_create(3, bad, Ls, 1.0, 0.3, 0, ctypes.byref(h)) == 1
    big = (ctypes.c_int * 3)(8, 2048, 8)
    assert L.bri17_op_create(3, big, Ls, 1.0, 0.3, 0, ctypes.byref(h)) == 2
    assert L.bri17_op_destroy(None) == 0
    assert L.bri17_apply_stiffness(None, None, None, None) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_no_device_is_reported():
    L = _lib.load()
    h = ctypes.c_void_p()
    shape = (ctypes.c_int * 2)(8, 8)
    Ls = (ctypes.c_double * 2)(1.0, 1.0)
    assert L.bri17_op_create(2, shape, Ls, 1.0, 0.3, 0, ctypes.byref(h)) == 7
    assert b"device" in L.bri17_last_error()


def test_host_grid_api_matches_reference_fixture(golden_modal):
    from bri17_gb300 import CartesianGrid
    for c in golden_modal:
        g = CartesianGrid(c["shape"], c["L"])
        nodes = np.array([g.get_cell_nodes(i) for i in range(g.size)])
        assert np.array_equal(nodes, c["nodes"])
    g = CartesianGrid((3, 4, 5), (1, 1, 1))
    assert g.get_node_at(2, 3, 4) == 59 and g.get_node_at(0, 1, 0) == 5


def test_pybri17_importable_under_the_reference_name():
    """``import pybri17`` (python/pybri17.cpp:98) finds the rebinding."""
    import pybri17

    from bri17_gb300 import pybri17 as inner
    assert pybri17.Hooke3f64 is inner.Hooke3f64
    assert pybri17.CartesianGrid2f64 is inner.CartesianGrid2f64
    assert pybri17.__version__ == "0.1" and pybri17.__author__ == "S. Brisard"


def test_pybri17_surface_and_contiguity_checks():
    from bri17_gb300 import pybri17
    assert pybri17.__author__ == "S. Brisard" and pybri17.__version__ == "0.1"
    g2 = pybri17.CartesianGrid2f64((3, 4), (1.1, 1.2))
    assert g2.dim == 2 and pybri17.CartesianGrid3f64.dim == 3
    assert g2.dtype == np.float64 and g2.size == 12 and g2.shape == (3, 4)
    assert g2.get_node_at(1, 2) == 6
    with pytest.raises(ValueError):
        pybri17._check_contiguous(np.zeros((2, 2), np.complex128), np.complex128)
    with pytest.raises(ValueError):
        pybri17._check_contiguous(np.zeros(8, np.complex128)[::2], np.complex128)
    with pytest.raises(TypeError):  # the reference would write into a temporary copy
        pybri17._check_contiguous(np.zeros(4, np.complex64), np.complex128)
    pybri17._check_contiguous(np.zeros(4, np.complex128), np.complex128)


_CPP_USES = r"""
#include <sstream>
#include "bri17/bri17_gpu.hpp"

template <typename T, int DIM>
int exercise(bool run) {
  if (!run) return 0;
  std::array<int, DIM> n{};
  std::array<T, DIM> L{};
  n.fill(8);
  L.fill(T(1));
  bri17::CartesianGrid<T, DIM> g(n, L);
  std::ostringstream os;
  os << g;
  int nodes = g.get_cell_nodes(0)[0];
  if constexpr (DIM == 2) nodes += g.get_node_at(1, 2); else nodes += g.get_node_at(1, 2, 3);
  bri17::Hooke<T, DIM> h(T(1), T(0.3), g);
  bri17::Hooke<T, DIM> h2(h);
  os << h << h2.repr();
  constexpr int sym = bri17::Hooke<T, DIM>::sym;
  int k[DIM] = {};
  std::complex<T> B[DIM], K[DIM * DIM], tau[sym], eta[sym];
  h.modal_strain_displacement(k, B);
  h.modal_stiffness(k, K);
  h.modal_eigenstress_to_opposite_strain(k, tau, eta);
  T* p = nullptr;
  h.apply_stiffness(p, p);
  h.apply_stiffness_host(p, p);
  h.apply_strain(p, p);
  h.eigenstress_rhs(p, p);
  h.eigenstress_to_opposite_strain(p, p);
  double* d = nullptr;
  bri17_cg_info info = h.cg_solve(d, d, 1e-8, 10, true);
  if constexpr (std::is_same<T, double>::value) h.set_float_pair(false);
  return nodes + info.iterations + (h.handle() != nullptr);
}

int main(int argc, char**) {
  const bool run = argc > 1000;  // compiled and linked, never run here
  return exercise<double, 2>(run) + exercise<double, 3>(run) + exercise<float, 2>(run) +
         exercise<float, 3>(run);
}
"""


def _nvcc():
    import os
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc absent")
    return nvcc


def test_cpp_host_api_compiles_and_links(tmp_path):
    """Every public member of include/bri17/bri17_gpu.hpp, for T = float and
    double and DIM = 2 and 3, compiles and resolves against the library; so
    does the GPU golden-test program (tests/cpp/test_bri17_gpu.cpp)."""
    import os
    import subprocess

    from conftest import REPO
    nvcc = _nvcc()
    inc, lib_dir = os.path.join(REPO, "include"), os.path.join(REPO, "bri17_gb300")
    link = ["-L", lib_dir, "-lbri17_gb300", f"-Xlinker=-rpath={lib_dir}"]
    src = tmp_path / "uses.cpp"
    src.write_text(_CPP_USES)
    for s, exe in ((str(src), tmp_path / "uses"),
                   (os.path.join(REPO, "tests", "cpp", "test_bri17_gpu.cpp"), tmp_path / "golden")):
        r = subprocess.run([nvcc, "-std=c++17", "-O1", "-I", inc, s, "-o", str(exe), *link],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("body,why", [
    ("bri17::Hooke<float, 3>* h = nullptr; h->set_float_pair(true);", "set_float_pair"),
    ("bri17::Hooke<long double, 3>* h = nullptr; (void)h->mu;", "float or double"),
])
def test_cpp_host_api_rejects_unsupported_types(tmp_path, body, why):
    """Float pairs exist only for FP64 handles, and the operator takes float
    or double fields only: both misuses fail to compile."""
    import os
    import subprocess

    from conftest import REPO
    src = tmp_path / "bad.cpp"
    src.write_text('#include "bri17/bri17_gpu.hpp"\nint main() { ' + body + " return 0; }\n")
    r = subprocess.run([_nvcc(), "-std=c++17", "-I", os.path.join(REPO, "include"),
                        "-c", str(src), "-o", str(tmp_path / "bad.o")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and why in r.stderr, r.stderr


def test_server_argument_validation_before_device():
    """bri17_server_* reject bad arguments and null handles before any
    device call (the server's poll writes at most `cap` results)."""
    L = _lib.load()
    s = ctypes.c_void_p()
    assert L.bri17_server_create(0, 8, ctypes.byref(s)) == 1
    assert L.bri17_server_create(1 << 30, 0, ctypes.byref(s)) == 1
    assert L.bri17_server_create(1 << 30, 257, ctypes.byref(s)) == 1
    assert L.bri17_server_create(1 << 30, 8, None) == 1
    n = ctypes.c_int()
    rid = ctypes.c_int64()
    shape = (ctypes.c_int * 3)(8, 8, 8)
    Ls = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    assert L.bri17_server_step(None, ctypes.byref(n)) == 1
    assert L.bri17_server_poll(None, None, 0, ctypes.byref(n)) == 1
    assert L.bri17_server_cancel(None, 0) == 1
    assert L.bri17_server_set_size_priority(None, 1) == 1
    assert L.bri17_server_submit(None, shape, Ls, 1.0, 0.3, None, None, 1e-8, 10,
                                 ctypes.byref(rid)) == 1
    assert L.bri17_server_destroy(None) == 0
    assert L.bri17_server_clock(None) == 0.0


def test_header_cites_the_reference_for_every_entry_point():
    """Every function the public header declares comes after a comment that
    either cites the reference interface it replaces (a file:line of the
    reference) or says that it has no reference counterpart.  A group of
    declarations shares the comment above the group."""
    import re
    with open(_lib.HEADER) as f:
        src = f.read()
    cite = re.compile(r"(bri17\.hpp|test_bri17\.cpp|pybri17\.cpp|demo\.py|version\.txt)"
                      r":\d+|:\d+-\d+|[Nn]o (reference )?counterpart|no counterpart")
    missing = []
    for name in _lib.declared_symbols():
        m = re.search(r"\b" + name + r"\s*\(", re.sub(r"/\*.*?\*/", lambda c: " " * len(
            c.group(0)), src, flags=re.S))
        assert m, name
        comments = list(re.finditer(r"/\*.*?\*/", src[:m.start()], flags=re.S))
        text = re.sub(r"\s*\n\s*\*?\s*", " ", comments[-1].group(0)) if comments else ""
        if not cite.search(text):
            missing.append(name)
    assert not missing, missing


def test_product_never_uses_the_oracle():
    """The package and the library never import, link or load the CPU oracle
    (no CPU fallback): no Python module of bri17_gb300 imports `oracle`, and
    the shared library's dynamic dependencies name no oracle library."""
    import ast
    import os
    import subprocess

    from conftest import REPO
    pkg = os.path.join(REPO, "bri17_gb300")
    for name in os.listdir(pkg):
        if not name.endswith(".py"):
            continue
        tree = ast.parse(open(os.path.join(pkg, name)).read())
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                assert not any(a.name.split(".")[0] == "oracle" for a in node.names), name
            elif isinstance(node, ast.ImportFrom):
                assert (node.module or "").split(".")[0] != "oracle", name
    r = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True)
    if r.returncode == 0:
        assert "oracle" not in r.stdout and "bri17_ref" not in r.stdout
