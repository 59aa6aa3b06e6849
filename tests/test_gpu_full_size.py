"""The solver configurations at their full sizes (the 256^3 eigenstress CG and
the anisotropic 512x512x128 one, with the workloads bench.py measures): the
mixed-precision CG's solution against the FP64 oracle's exact per-mode solve
(include/bri17/bri17.hpp:308-355, over the half spectrum)."""
import os

import numpy as np
import pytest

from gpu_helpers import rel_l2, to_dev
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _solve_and_compare(w, tau, tol):
    from bri17_gb300 import CartesianGrid, Hooke
    h = Hooke(w["mu"], w["nu"], CartesianGrid(w["shape"], w["L"]))
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=tol, mode="mixed")
    assert info["status"] == 0 and info["rel_residual"] <= tol, info
    O.set_num_threads(os.cpu_count() or 1)
    ho = O.Hooke(w["mu"], w["nu"], O.Grid(w["shape"], w["L"]))
    x_ref = O.eigenstress_solve_half(ho, tau, workers=os.cpu_count() or 1)
    return rel_l2(x.cpu().numpy(), x_ref), info


def test_cg_256_cubed_reaches_1e_8_against_the_oracle():
    """256^3, nu = 0.3, tau ~ N(0, 1) (seed 2): at the residual tolerance
    the benchmark's accuracy-targeted run uses (1e-11), the mixed CG lands
    within 1e-8 of the oracle (measured 1.8e-9 to 2.1e-9)."""
    import bench
    w = bench.WORKLOAD_CG
    err, info = _solve_and_compare(w, bench.tau_normal(w["shape"], w["seed"]), bench.ACC_TOL_256)
    assert err <= 1e-8, (err, info)


def test_cg_anisotropic_512x512x128_against_the_oracle():
    """512x512x128 with h = (1/512, 1/512, 1/1024), nu = 0.35, two inclusion
    columns plus noise (seed 4), residual 1e-8: the mixed CG's solution is
    within 1e-8 of the oracle (measured 5.8e-9 to 6.6e-9; the FP64 CG's 1.7e-9)."""
    import bench
    w = bench.WORKLOAD_ANISO
    err, info = _solve_and_compare(w, bench.tau_inclusions(w["shape"], w["L"], w["seed"]), 1e-8)
    assert err <= 1e-8, (err, info)
