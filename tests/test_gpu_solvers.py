"""GPU parity of the eigenstress right-hand side, the strain map and the CG
solvers against the oracle (the exact per-mode solve of
include/bri17/bri17.hpp:308-355)."""
import numpy as np
import pytest

from gpu_helpers import mean_free_normal, pair, rel_l2, to_dev
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,L", [((12, 10), (1.0, 1.2)), ((3, 4, 5), (3.3, 4.8, 6.5)),
                                     ((16, 12, 10), (1.0, 0.8, 1.1)), ((9, 14, 7), (1., 1., 1.))])
def test_eigenstress_rhs_matches_oracle(shape, L):
    h, ho = pair(shape, L, 1.0, 0.3)
    sym = 3 if len(shape) == 2 else 6
    tau = np.random.default_rng(7).standard_normal((sym,) + shape)
    b = h.eigenstress_rhs(to_dev(tau)).cpu().numpy()
    assert rel_l2(b, O.eigenstress_rhs(ho, tau)) <= 1e-12
    assert np.abs(b.reshape(len(shape), -1).mean(axis=1)).max() <= 1e-14 * np.abs(b).max()


@pytest.mark.parametrize("shape,L", [((12, 10), (1.0, 1.2)), ((16, 12, 10), (1.0, 0.8, 1.1)),
                                     ((5, 6, 7), (1.0, 1.0, 1.0))])
def test_strain_matches_oracle(shape, L):
    h, ho = pair(shape, L, 1.0, 0.3)
    u = np.random.default_rng(8).standard_normal((len(shape),) + shape)
    eps = h.apply_strain(to_dev(u)).cpu().numpy()
    assert rel_l2(eps, O.apply_strain(ho, u)) <= 1e-12


@pytest.mark.parametrize("mode", ["plain", "mixed", "mixed_restart"])
@pytest.mark.parametrize("shape,nu", [((32, 32, 32), 0.3), ((24, 20, 16), 0.45), ((48, 40), 0.3)])
def test_cg_matches_modal_direct_solve(mode, shape, nu):
    """CG to 1e-10 relative residual vs the exact FP64 per-mode solve;
    error <= kappa * residual bounds the difference."""
    L = (1.0,) * len(shape)
    h, ho = pair(shape, L, 1.0, nu)
    sym = 3 if len(shape) == 2 else 6
    tau = np.random.default_rng(2).standard_normal((sym,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=1e-10, mode=mode)
    assert info["status"] == 0, info
    assert info["rel_residual"] <= 1e-10
    x_ref = O.eigenstress_solve(ho, tau)
    assert rel_l2(x.cpu().numpy(), x_ref) <= 1e-6
    # The returned residual is the FP64 one.
    r = b - h.apply_stiffness(x)
    assert float(r.norm() / b.norm()) <= 1.01e-10


def test_cg_edge_cases():
    import torch
    h, _ = pair((8, 8, 8), (1.0, 1.0, 1.0), 1.0, 0.3)
    zero = torch.zeros((3, 8, 8, 8), dtype=torch.float64, device="cuda")
    x, info = h.cg_solve(zero, tol=1e-8)
    assert info["status"] == 0 and float(x.abs().max()) == 0.0
    tau = np.random.default_rng(3).standard_normal((6, 8, 8, 8))
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=1e-14, max_iterations=3, raise_on_failure=False)
    assert info["status"] == 5  # not converged
    bad = b.clone()
    bad[0, 0, 0, 0] = float("nan")
    x, info = h.cg_solve(bad, tol=1e-8, raise_on_failure=False)
    assert info["status"] == 6  # breakdown
    # The handle stays usable after a breakdown.
    x, info = h.cg_solve(b, tol=1e-8)
    assert info["status"] == 0


def test_cg_warm_start_and_material_change():
    h, ho = pair((16, 16, 16), (1.0, 1.0, 1.0), 1.0, 0.3)
    tau = np.random.default_rng(4).standard_normal((6, 16, 16, 16))
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=1e-6)
    x2, info2 = h.cg_solve(b, x0=x, tol=1e-10)
    assert info2["iterations"] < 200 and info2["rel_residual"] <= 1e-10
    for bad_x0 in (x.cpu(), x.float(), x[:2]):  # host memory, FP32, wrong size
        with pytest.raises(ValueError):
            h.cg_solve(b, x0=bad_x0)
    h.set_material(2.0, 0.2)
    ho2 = O.Hooke(2.0, 0.2, ho.grid)
    x3, info3 = h.cg_solve(b, tol=1e-10, mode="mixed")
    assert rel_l2(x3.cpu().numpy(), O.eigenstress_solve(ho2, tau)) <= 1e-6


@pytest.mark.parametrize("shape,nu", [((32, 32, 32), 0.3), ((48, 40), 0.45)])
def test_mixed_reliable_keeps_fp64_iteration_count(shape, nu):
    """Reliable updates keep the Krylov space: the mixed solve needs about as
    many operator applications as plain FP64 CG (a solve that resumed with
    a stale search direction after an update would need far more)."""
    L = (1.0,) * len(shape)
    h, _ = pair(shape, L, 1.0, nu)
    sym = 3 if len(shape) == 2 else 6
    tau = np.random.default_rng(12).standard_normal((sym,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    _, plain = h.cg_solve(b, tol=1e-10, mode="plain")
    _, mixed = h.cg_solve(b, tol=1e-10, mode="mixed")
    assert mixed["status"] == 0 and plain["status"] == 0
    assert mixed["iterations"] <= 1.3 * plain["iterations"] + 16, (mixed, plain)
    assert mixed["outer_iterations"] >= 2


@pytest.mark.parametrize("shape", [(12, 10), (16, 12, 10), (5, 6, 7)])
def test_f32_handle_strain_and_rhs(shape):
    """The strain map and the eigenstress right-hand side on an FP32 handle
    (generic and power-of-two paths) agree with the FP64 oracle to FP32
    accuracy."""
    import torch
    L = (1.0,) * len(shape)
    h, ho = pair(shape, L, 1.2, 0.25, precision="f32")
    rng = np.random.default_rng(13)
    sym = 3 if len(shape) == 2 else 6
    u = rng.standard_normal((len(shape),) + shape)
    tau = rng.standard_normal((sym,) + shape)
    eps = h.apply_strain(to_dev(u, torch.float32)).double().cpu().numpy()
    b = h.eigenstress_rhs(to_dev(tau, torch.float32)).double().cpu().numpy()
    assert rel_l2(eps, O.apply_strain(ho, u)) <= 2e-5
    assert rel_l2(b, O.eigenstress_rhs(ho, tau)) <= 2e-5


def test_handle_info_and_modal_batch_on_f32_handle(golden_modal):
    import ctypes

    from bri17_gb300 import _lib
    c = golden_modal[3]
    h, _ = pair(c["shape"], c["L"], c["mu"], c["nu"], precision="f32")
    K = h.modal_stiffness_batch(c["k"]).cpu().numpy().reshape(len(c["k"]), -1)
    inr = np.all((c["k"] >= 0) & (c["k"] < np.array(c["shape"])), axis=1)
    # The per-mode API computes in FP64 whatever the handle's field precision.
    assert np.array_equal(K[inr].view(np.float64), c["K"][inr].view(np.float64))
    size, ws = ctypes.c_int64(), ctypes.c_int64()
    assert _lib.load().bri17_op_info(h.handle, ctypes.byref(size), ctypes.byref(ws)) == 0
    n = c["shape"]
    assert size.value == int(np.prod(n))
    assert ws.value == 3 * n[0] * n[1] * (n[2] // 2 + 1) * 8


def test_wrong_device_and_dtype_are_rejected():
    import torch

    from bri17_gb300._lib import Bri17Error
    h, _ = pair((8, 8, 8), (1.0, 1.0, 1.0), 1.0, 0.3)
    with pytest.raises(TypeError):
        h.apply_stiffness(torch.zeros((3, 8, 8, 8), dtype=torch.float32, device="cuda"))
    with pytest.raises(ValueError):
        h.apply_stiffness(torch.zeros((3, 8, 8, 7), dtype=torch.float64, device="cuda"))
    with pytest.raises(Bri17Error):
        h.set_material(1.0, 0.5)


# Field form of Hooke::modal_eigenstress_to_opposite_strain (the direct
# solution of the eigenstress problem, python/demo.py's per-mode loop on the
# whole spectrum) against the oracle: FP64 at the operator's 1e-12 bound,
# FP32 at its 2e-5; 2D and 3D, odd and power-of-two sides.
OPP_SHAPES = [
    ((16, 12), (1.0, 0.75), 1.0, 0.3),
    ((8, 8, 8), (1.0, 1.0, 1.0), 1.0, 0.25),
    ((7, 10, 6), (1.0, 2.0, 0.5), 0.7, 0.45),
    ((32, 16, 24), (1.0, 1.0, 1.0), 1.3, 0.1),
]


@pytest.mark.parametrize("shape,L,mu,nu", OPP_SHAPES)
def test_opposite_strain_field_matches_oracle(shape, L, mu, nu):
    from gpu_helpers import pair, rel_l2, to_dev
    sym = 3 if len(shape) == 2 else 6
    rng = np.random.default_rng(31)
    tau = rng.standard_normal((sym,) + shape)
    for precision, tol in (("f64", 1e-12), ("f32", 2e-5)):
        h, ho = pair(shape, L, mu, nu, precision=precision)
        eta_ref = O.eigenstress_opposite_strain(ho, tau)
        t = to_dev(tau.astype(np.float64 if precision == "f64" else np.float32))
        eta = h.eigenstress_to_opposite_strain(t).cpu().numpy().astype(np.float64)
        assert rel_l2(eta, eta_ref) <= tol, precision


@pytest.mark.parametrize("mode", ["mixed", "plain"])
def test_cg_reaches_1e_8_error_against_the_oracle(mode):
    """The solver accuracy target: at a residual tolerance of 1e-11, the
    mixed-precision CG (FP32 operator, FP64 reliable updates) and the FP64 CG
    both land within 1e-8 relative l2 of the FP64 oracle's exact modal
    solution (kappa ~ 3e3 at 96^3; measured 6e-10 and 1.4e-10)."""
    shape = (96, 96, 96)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    tau = np.random.default_rng(2).standard_normal((6,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=1e-11, mode=mode)
    assert info["status"] == 0 and info["rel_residual"] <= 1e-11, info
    x_ref = O.eigenstress_solve_half(ho, tau, workers=4)
    assert rel_l2(x.cpu().numpy(), x_ref) <= 1e-8


def test_cg_on_a_float_pair_handle():
    """With float pairs on, the plain CG's operator applications run in
    float pairs: same accuracy against the oracle as the FP64-pipe solver,
    about the same iteration count.  (The mixed CG's FP64 residuals run in
    float pairs on this grid either way.)"""
    shape = (64, 64, 128)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    tau = np.random.default_rng(10).standard_normal((6,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    x_ref = O.eigenstress_solve_half(ho, tau, workers=4)
    res = {}
    for fp in (False, True):
        h.set_float_pair(fp)
        for mode in ("plain", "mixed"):
            x, info = h.cg_solve(b, tol=1e-11, mode=mode)
            assert info["status"] == 0 and info["rel_residual"] <= 1e-11, (fp, mode, info)
            res[(fp, mode)] = (rel_l2(x.cpu().numpy(), x_ref), info["iterations"])
    h.set_float_pair(False)
    for mode in ("plain", "mixed"):
        e64, it64 = res[(False, mode)]
        efp, itfp = res[(True, mode)]
        assert efp <= max(2 * e64, 1e-9), (mode, efp, e64)
        assert itfp <= 1.1 * it64 + 8, (mode, itfp, it64)


@pytest.mark.parametrize("shape,L", [((32, 32, 32), (1.0, 1.0, 1.0)),
                                     ((64, 32, 16), (1.0, 0.5, 0.25)),
                                     ((16, 8, 64), (1.0, 1.0, 2.0))])
def test_mixed_cg_matches_oracle_and_is_deterministic(shape, L):
    """Mixed CG on power-of-two 3D grids of unequal axes: same accuracy as
    the FP64 solver against the oracle, and bit-identical solutions from two
    solves (fixed-order reductions, no atomics in any sum)."""
    h, ho = pair(shape, L, 1.0, 0.3)
    tau = np.random.default_rng(9).standard_normal((6,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    x1, i1 = h.cg_solve(b, tol=1e-10, mode="mixed")
    x2, i2 = h.cg_solve(b, tol=1e-10, mode="mixed")
    xp, ip = h.cg_solve(b, tol=1e-10, mode="plain")
    assert i1["status"] == 0 and i1["rel_residual"] <= 1e-10, i1
    assert bool((x1 == x2).all()) and i1["iterations"] == i2["iterations"]
    x_ref = O.eigenstress_solve(ho, tau)
    e1 = rel_l2(x1.cpu().numpy(), x_ref)
    ep = rel_l2(xp.cpu().numpy(), x_ref)
    assert e1 <= max(4 * ep, 1e-8), (e1, ep)
    # About as many iterations as plain CG (reliable updates keep p).
    assert i1["iterations"] <= 1.3 * ip["iterations"] + 16, (i1, ip)


@pytest.mark.parametrize("shape", [(64, 64, 128), (128, 32, 16)])
def test_fp32_cg_with_pq_in_the_stiffness_pass(shape):
    """With the TMA-staged axis-0 form, the FP32 CG sums p.Kp by Parseval in
    the stiffness pass (no separate pass over p and q); with the staged form
    it runs the separate reduction.  Both converge alike, land equally close
    to the oracle, and repeat bit for bit (fixed-order reductions)."""
    L = (1.0, 0.9, 1.1)
    h32, ho = pair(shape, L, 1.0, 0.3, precision="f32")
    h64, _ = pair(shape, L, 1.0, 0.3)
    tau = np.random.default_rng(11).standard_normal((6,) + shape)
    b = h64.eigenstress_rhs(to_dev(tau))
    x_ref = O.eigenstress_solve_half(ho, tau, workers=4)
    res = {}
    for form in ("tma", "staged"):
        h32.fused_form = form
        x1, i1 = h32.cg_solve(b, tol=1e-5, mode="plain")
        x2, i2 = h32.cg_solve(b, tol=1e-5, mode="plain")
        assert i1["status"] == 0 and i1["rel_residual"] <= 1e-5, (form, i1)
        assert bool((x1 == x2).all()) and i1["iterations"] == i2["iterations"], form
        res[form] = (rel_l2(x1.cpu().numpy(), x_ref), i1["iterations"])
    (et, it_t), (es, it_s) = res["tma"], res["staged"]
    assert et <= max(2 * es, 1e-4), (et, es)
    assert abs(it_t - it_s) <= 0.1 * it_s + 4, (it_t, it_s)
