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
