"""bri17_apply_stiffness_noalloc: the operator for callers that cannot
allocate device memory (a plugin whose host owns every allocation, a fixed
device-memory budget, or code that must not let cudaMalloc synchronise the
device).  It must give the allocating entry point's results, through the C
ABI, on consecutive calls that reuse its one fixed scratch array.

This file sorts last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from bri17_gb300 import _lib

TOL_F64 = 1e-12  # relative l2, the FP64 operator tolerance of the parity tests


def _noalloc(shape, L, mu, nu, u, f):
    Lib = _lib.load()
    dim = len(shape)
    return Lib.bri17_apply_stiffness_noalloc(
        dim, (ctypes.c_int * dim)(*shape), (ctypes.c_double * dim)(*L), mu, nu,
        ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(f.data_ptr()), None)


def test_noalloc_rejects_grids_beyond_its_scratch():
    """256^3 needs more than the fixed 64 MiB scratch: refused before any
    device work, with a clear message."""
    Lib = _lib.load()
    shape = (256, 256, 256)
    rc = Lib.bri17_apply_stiffness_noalloc(
        3, (ctypes.c_int * 3)(*shape), (ctypes.c_double * 3)(1, 1, 1), 1.0, 0.3,
        ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == 2
    assert b"64 MiB" in Lib.bri17_last_error()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    import torch

    from bri17_gb300 import CartesianGrid, Hooke
    rng = np.random.default_rng(21)
    # The last two cases follow the 128^3 call, so they run on a scratch
    # array whose tables and spectrum a larger grid left behind.
    cases = [((24, 20, 18), (1.0, 0.8, 1.2), 1.3, 0.3),
             ((64, 48), (1.0, 0.75), 0.8, 0.2),
             ((128, 128, 128), (1.0, 1.0, 1.0), 1.0, 0.25),
             ((24, 20, 18), (1.0, 0.8, 1.2), 1.3, 0.3),
             ((30, 22), (0.9, 1.1), 1.7, 0.35)]
    for shape, L, mu, nu in cases:
        h = Hooke(mu, nu, CartesianGrid(shape, L))
        for call in range(2):
            u = torch.from_numpy(rng.standard_normal((len(shape),) + shape)).cuda()
            f_ref = h.apply_stiffness(u)
            f = torch.full_like(u, float("nan"))
            assert _noalloc(shape, L, mu, nu, u, f) == 0, _lib.load().bri17_last_error()
            torch.cuda.synchronize()
            err = float((f - f_ref).norm() / f_ref.norm())
            assert err <= TOL_F64, (shape, call, err)
