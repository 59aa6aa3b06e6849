"""GPU parity of the periodic stiffness operator (CUDA path through the C
ABI) against the oracle and the reference's golden element matrices."""
import numpy as np
import pytest

from gpu_helpers import mean_free_normal, pair, rel_l2, to_dev
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# Floating-point tolerances (relative l2, FP64 / FP32 operator vs oracle).
TOL_F64 = 1e-12
TOL_F32 = 2e-5


def _dense_from_gpu(fn, ncols, nrows, dtype):
    import torch
    M = np.empty((nrows, ncols))
    e = torch.zeros(ncols, dtype=dtype, device="cuda")
    for j in range(ncols):
        e.zero_()
        e[j] = 1.0
        M[:, j] = fn(e).reshape(-1).double().cpu().numpy()
    return M


@pytest.mark.parametrize("case_index", [0, 1, 2, 3])
def test_golden_element_matrices(golden_elements, case_index):
    """tests/test_bri17.cpp:335-605 on the GPU: K (B) extracted by unit
    vectors equals the assembly of the Maxima element matrix,
    |a - e| <= 1e-15 |e| + 1e-14."""
    import torch
    g = golden_elements
    case = g["cases"][case_index]
    h, ho = pair(case["shape"], case["L"], g["mu"], g["nu"])
    grid = ho.grid
    E = np.array(case["values"]).reshape(case["rows"], case["cols"])
    n = grid.dim * grid.size
    if case["kind"] == "K":
        expected = O.assemble_stiffness(grid, E)
        actual = _dense_from_gpu(
            lambda e: h.apply_stiffness(e.reshape((grid.dim,) + grid.shape)), n, n,
            torch.float64)
    else:
        sym = 3 if grid.dim == 2 else 6
        expected = O.assemble_strain_displacement(grid, E)
        actual = _dense_from_gpu(
            lambda e: h.apply_strain(e.reshape((grid.dim,) + grid.shape)), n,
            sym * grid.size, torch.float64)
    err = np.abs(actual - expected)
    tol = g["rtol"] * np.abs(expected) + g["atol"]
    assert np.all(err <= tol), f"max excess {(err - tol).max()}"


SHAPES = [
    ((64, 64), (1.0, 1.0), 1.0, 0.3),          # 2D Q4 64x64 case
    ((3, 4), (3.3, 4.8), 5.6, 0.3),
    ((5, 7), (1.0, 2.0), 2.0, 0.1),
    ((6, 10), (0.5, 1.5), 1.0, 0.45),
    ((48, 96), (1.0, 2.0), 0.7, 0.2),
    ((1, 8), (1.0, 1.0), 1.0, 0.3),
    ((3, 4, 5), (3.3, 4.8, 6.5), 5.6, 0.3),
    ((8, 8, 8), (1.0, 1.0, 1.0), 1.0, 0.25),
    ((6, 10, 8), (1.0, 2.5, 0.75), 1.7, 0.45),
    ((12, 9, 7), (1.0, 1.0, 0.125), 0.5, 0.1),
    ((32, 48, 20), (1.0, 1.5, 0.6), 1.0, 0.3),
    ((7, 11, 13), (1.0, 1.0, 1.0), 1.0, 0.3),   # generic odd radices
    ((14, 21, 22), (2.0, 1.0, 1.0), 1.2, 0.35),
    ((96, 32, 64), (3.0, 1.0, 2.0), 1.0, 0.3),
    ((16, 4, 1), (1.0, 1.0, 1.0), 1.0, 0.3),    # degenerate last axis
    ((1024, 16), (1.0, 0.5), 1.0, 0.3),          # register-resident engine, long axes
    ((16, 1024, 8), (1.0, 2.0, 0.5), 0.9, 0.2),
    ((512, 8, 32), (2.0, 1.0, 1.0), 1.1, 0.4),
    ((8, 16, 16), (1.0, 1.0, 1.0), 1.0, 0.3),
    ((256, 64, 128), (1.0, 0.25, 0.5), 1.0, 0.3),
    ((1, 6, 10), (1.0, 1.0, 1.0), 1.0, 0.3),    # degenerate first axis
    ((8, 256, 64), (1.0, 2.0, 0.5), 1.0, 0.3),   # axis-1 lengths of the 16-element FP32 pass
    ((4, 512, 32), (1.0, 1.0, 1.0), 0.8, 0.2),
    # lengths 3 * 2^k on the twelve-element engine: every axis and the rows
    ((96, 96, 96), (1.0, 1.0, 1.0), 1.0, 0.3),
    ((24, 192, 48), (0.5, 2.0, 1.0), 1.3, 0.35),
    ((192, 24, 384), (2.0, 0.25, 4.0), 0.9, 0.2),
    ((48, 3, 96), (1.0, 1.0, 1.0), 1.0, 0.3),
]


@pytest.mark.parametrize("shape,L,mu,nu", SHAPES)
def test_operator_matches_oracle_f64(shape, L, mu, nu):
    h, ho = pair(shape, L, mu, nu)
    rng = np.random.default_rng(0)
    u = mean_free_normal(rng, len(shape), shape)
    f = h.apply_stiffness(to_dev(u)).cpu().numpy()
    f_ref = O.apply_stiffness(ho, u)
    assert rel_l2(f, f_ref) <= TOL_F64


@pytest.mark.parametrize("shape,L,mu,nu", SHAPES)
def test_operator_matches_oracle_f32(shape, L, mu, nu):
    import torch
    h, ho = pair(shape, L, mu, nu, precision="f32")
    rng = np.random.default_rng(1)
    u = mean_free_normal(rng, len(shape), shape).astype(np.float32)
    f = h.apply_stiffness(to_dev(u)).cpu().numpy().astype(np.float64)
    f_ref = O.apply_stiffness(ho, u.astype(np.float64))
    assert rel_l2(f, f_ref) <= TOL_F32


def test_operator_128_cubed_matches_oracle():
    """3D 128^3, h = 1/128, mu = 1, nu = 0.25, u ~ N(0,1) seeded, mean-free."""
    shape = (128, 128, 128)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.25)
    rng = np.random.default_rng(1)
    u = mean_free_normal(rng, 3, shape)
    f = h.apply_stiffness(to_dev(u)).cpu().numpy()
    assert rel_l2(f, O.apply_stiffness(ho, u)) <= TOL_F64


def test_operator_properties():
    """Symmetry, rigid translations in the null space, linearity, aliasing,
    bitwise determinism."""
    import torch
    shape = (24, 20, 18)
    h, _ = pair(shape, (1.0, 0.8, 1.2), 1.3, 0.3)
    rng = np.random.default_rng(2)
    u = to_dev(rng.standard_normal((3,) + shape))
    v = to_dev(rng.standard_normal((3,) + shape))
    Ku, Kv = h.apply_stiffness(u), h.apply_stiffness(v)
    a, b = float((v * Ku).sum()), float((u * Kv).sum())
    assert abs(a - b) <= 1e-12 * abs(a)
    c = torch.ones((3,) + shape, dtype=torch.float64, device="cuda")
    c[1] *= -2.5
    assert float(h.apply_stiffness(c).abs().max()) <= 1e-12 * float(Ku.abs().max())
    w = h.apply_stiffness(2.0 * u - 3.0 * v)
    assert float((w - (2.0 * Ku - 3.0 * Kv)).norm() / w.norm()) <= 1e-13
    again = h.apply_stiffness(u)
    assert torch.equal(again, Ku)
    alias = u.clone()
    h.apply_stiffness(alias, out=alias)
    assert torch.equal(alias, Ku)


def test_host_buffer_entry_point():
    shape = (16, 12, 10)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    rng = np.random.default_rng(4)
    u = rng.standard_normal((3,) + shape)
    f = h.apply_stiffness_host(u)
    assert rel_l2(f, O.apply_stiffness(ho, u)) <= TOL_F64
    assert np.array_equal(f, h.apply_stiffness(to_dev(u)).cpu().numpy())


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_host_buffer_page_locked_in_place(precision):
    """Page-locked host tensors: the passes read u and write f in host memory
    (no staging copies); same values as the device entry point, bit for
    bit, including in place (f aliasing u)."""
    import torch
    shape = (32, 24, 20)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3, precision=precision)
    dt = torch.float64 if precision == "f64" else torch.float32
    rng = np.random.default_rng(5)
    u = torch.from_numpy(rng.standard_normal((3,) + shape)).to(dt).pin_memory()
    f = h.apply_stiffness_host(u)
    assert f.is_pinned() and not f.is_cuda
    ref = h.apply_stiffness(u.cuda()).cpu()
    assert torch.equal(f, ref)
    tol = TOL_F64 if precision == "f64" else TOL_F32
    assert rel_l2(f.double().numpy(), O.apply_stiffness(ho, u.double().numpy())) <= tol
    import ctypes
    from bri17_gb300 import _lib
    w = u.clone().pin_memory()
    assert _lib.load().bri17_apply_stiffness_host(
        h.handle, ctypes.c_void_p(w.data_ptr()), ctypes.c_void_p(w.data_ptr()), None) == 0
    assert torch.equal(w, ref)


def test_modal_batch_matches_reference_fixture(golden_modal):
    """Batched Hooke::modal_stiffness equals the reference header's output
    bit for bit for in-range k; B and out-of-range K to 1e-15."""
    for c in golden_modal:
        h, _ = pair(c["shape"], c["L"], c["mu"], c["nu"])
        k = c["k"]
        dim = len(c["shape"])
        K = h.modal_stiffness_batch(k).cpu().numpy().reshape(len(k), -1)
        B = h.modal_strain_displacement_batch(k).cpu().numpy()
        inr = np.all((k >= 0) & (k < np.array(c["shape"])), axis=1)
        assert np.array_equal(K[inr].view(np.float64), c["K"][inr].view(np.float64))
        scale = np.abs(c["K"]).max()
        assert np.abs(K - c["K"]).max() <= 1e-15 * scale * 4
        bscale = np.abs(c["B"]).max()
        assert np.abs(B - c["B"]).max() <= 1e-15 * bscale * 4


def test_modal_eigenstress_batch_matches_oracle():
    shape, L = (6, 10, 8), (1.0, 2.5, 0.75)
    h, ho = pair(shape, L, 1.7, 0.45)
    rng = np.random.default_rng(6)
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    k = np.stack([x.ravel() for x in grids], 1).astype(np.intc)
    tau = rng.standard_normal((len(k), 6)) + 1j * rng.standard_normal((len(k), 6))
    eta = h.modal_eigenstress_to_opposite_strain_batch(k, tau).cpu().numpy()
    ref = np.array([ho.modal_eigenstress_to_opposite_strain(kk, t) for kk, t in zip(k, tau)])
    assert np.abs(eta - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.all(eta[0] == 0)


def test_pybri17_per_mode_methods(golden_modal):
    from bri17_gb300 import pybri17
    c = golden_modal[1]
    grid = pybri17.CartesianGrid3f64(tuple(c["shape"]), tuple(c["L"]))
    h = pybri17.Hooke3f64(c["mu"], c["nu"], grid)
    for i in (0, 7, 33, 59):
        K = np.zeros(9, dtype=np.complex128)
        B = np.zeros(3, dtype=np.complex128)
        h.modal_stiffness_matrix(c["k"][i], K)
        h.modal_strain_displacement(c["k"][i], B)
        assert np.array_equal(K, c["K"][i])
        assert np.abs(B - c["B"][i]).max() <= 4e-15 * np.abs(c["B"]).max()
    with pytest.raises(ValueError):
        h.modal_stiffness_matrix(c["k"][0], np.zeros((3, 3), np.complex128))


@pytest.mark.parametrize("case", [0, 1])
def test_per_mode_host_entry_points_match_device_batches(golden_modal, case):
    """bri17_modal_*_host (host buffers, staging kept by the handle) give the
    device batch entry points' values -- K and B bit for bit -- on batches of
    one and of many modes, through the top-level ``pybri17`` name too."""
    import ctypes
    import time

    import pybri17
    from bri17_gb300 import _lib
    c = golden_modal[case]
    dim = len(c["shape"])
    grid = (pybri17.CartesianGrid2f64 if dim == 2 else pybri17.CartesianGrid3f64)(
        tuple(c["shape"]), tuple(c["L"]))
    h = (pybri17.Hooke2f64 if dim == 2 else pybri17.Hooke3f64)(c["mu"], c["nu"], grid)
    L = _lib.load()
    k = np.ascontiguousarray(c["k"], dtype=np.intc)
    n = k.shape[0]
    K = np.empty((n, dim * dim), np.complex128)
    B = np.empty((n, dim), np.complex128)
    vp = ctypes.c_void_p
    assert L.bri17_modal_stiffness_host(h.handle, vp(k.ctypes.data), n, vp(K.ctypes.data)) == 0
    assert L.bri17_modal_strain_displacement_host(h.handle, vp(k.ctypes.data), n,
                                                  vp(B.ctypes.data)) == 0
    assert np.array_equal(K, h.modal_stiffness_batch(k).cpu().numpy().reshape(n, -1))
    assert np.array_equal(B, h.modal_strain_displacement_batch(k).cpu().numpy())
    inr = np.all((k >= 0) & (k < np.array(c["shape"])), axis=1)  # the fixture's in-range k
    assert np.array_equal(K[inr], c["K"].reshape(n, -1)[inr])
    sym = 3 if dim == 2 else 6
    rng = np.random.default_rng(12)
    tau = rng.standard_normal((n, sym)) + 1j * rng.standard_normal((n, sym))
    eta = np.empty_like(tau)
    assert L.bri17_modal_eigenstress_to_opposite_strain_host(
        h.handle, vp(k.ctypes.data), n, vp(tau.ctypes.data), vp(eta.ctypes.data)) == 0
    eta_dev = h.modal_eigenstress_to_opposite_strain_batch(k, tau).cpu().numpy()
    # Same kernel, same inputs: identical, including the NaN a k that wraps
    # to 0 without being 0 produces (K(k) = 0 there).
    assert np.array_equal(eta, eta_dev, equal_nan=True)
    ho = O.Hooke(c["mu"], c["nu"], O.Grid(c["shape"], c["L"]))
    ref = np.array([ho.modal_eigenstress_to_opposite_strain(kk, t)
                    for kk, t in zip(k[inr], tau[inr])])
    assert np.abs(eta[inr] - ref).max() <= 1e-13 * np.abs(ref).max()
    # One mode at a time through the reference's per-mode surface.
    Ki = np.zeros(dim * dim, np.complex128)
    etai = np.zeros(sym, np.complex128)
    t0 = time.perf_counter()
    for i in range(n):
        h.modal_stiffness_matrix(k[i], Ki)
        assert np.array_equal(Ki, K[i])
    per_call_us = (time.perf_counter() - t0) / n * 1e6
    i3 = int(np.argwhere(inr)[3][0])
    h.modal_eigenstress_to_opposite_strain(k[i3], np.ascontiguousarray(tau[i3]), etai)
    assert np.array_equal(etai, eta[i3])
    print(f"per-mode call through pybri17: {per_call_us:.1f} us")


# Every form of the FP32 axis-0 stiffness pass against the oracle: register-
# resident, shared-memory staged and TMA-staged (tensor copies of whole
# tiles; 3D with an even shape[1]).  Shapes cover partial last tiles (P not a
# multiple of the tile's lines), the 256-row box split (n0 = 512, 1024) and
# one where the TMA form declines (odd shape[1]) and falls back.
FORM_SHAPES = [
    ((16, 8, 8), (1.0, 1.0, 1.0), 1.0, 0.3),
    ((64, 10, 6), (1.0, 2.0, 0.5), 0.8, 0.2),
    ((128, 16, 30), (1.0, 1.0, 1.0), 1.2, 0.35),
    ((256, 12, 16), (1.0, 0.5, 0.5), 1.0, 0.3),
    ((512, 8, 14), (2.0, 1.0, 1.0), 1.1, 0.4),
    ((1024, 4, 8), (1.0, 1.0, 1.0), 0.9, 0.25),
    ((64, 9, 8), (1.0, 1.0, 1.0), 1.0, 0.3),
]


@pytest.mark.parametrize("shape,L,mu,nu", FORM_SHAPES)
def test_fused_forms_f32_match_oracle(shape, L, mu, nu):
    import torch
    from bri17_gb300 import wait_timeouts
    h, ho = pair(shape, L, mu, nu, precision="f32")
    assert h.fused_form in h.FUSED_FORMS
    rng = np.random.default_rng(11)
    u = mean_free_normal(rng, 3, shape).astype(np.float32)
    f_ref = O.apply_stiffness(ho, u.astype(np.float64))
    ud = to_dev(u)
    assert wait_timeouts() >= 0
    outs = {}
    for form in h.FUSED_FORMS:
        h.fused_form = form
        outs[form] = h.apply_stiffness(ud)
        torch.cuda.synchronize()
        f = outs[form].cpu().numpy().astype(np.float64)
        assert rel_l2(f, f_ref) <= TOL_F32, form
    assert wait_timeouts() == 0
    for form in ("staged", "tma", "tma_registers"):
        d = float((outs[form] - outs["registers"]).norm() / outs["registers"].norm())
        assert d <= 1e-6, form


def test_tma_form_64_cubed():
    """The TMA form at 64^3 (full tiles, one box per component)."""
    from bri17_gb300 import wait_timeouts
    shape = (64, 64, 64)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3, precision="f32")
    h.fused_form = "tma"
    rng = np.random.default_rng(12)
    u = mean_free_normal(rng, 3, shape).astype(np.float32)
    f = h.apply_stiffness(to_dev(u)).cpu().numpy().astype(np.float64)
    assert rel_l2(f, O.apply_stiffness(ho, u.astype(np.float64))) <= TOL_F32
    assert wait_timeouts() == 0


# Float-pair arithmetic on FP64 handles (hi + lo floats, 48-bit
# significands): the FP64 parity bound of 1e-12 against the oracle, both
# axis-0 forms, field magnitudes far from 1, host buffers, rejected grids.
FLOAT_PAIR_SHAPES = [
    ((64, 64, 128), (1.0, 1.0, 1.0), 1.0, 0.25),
    ((128, 128, 128), (1.0, 1.0, 1.0), 1.0, 0.25),
    ((64, 256, 256), (1.0, 2.0, 0.5), 0.8, 0.35),
    ((512, 64, 128), (1.0, 1.0, 0.125), 1.0, 0.35),
    ((64, 128), (1.0, 1.0), 1.0, 0.3),
    ((512, 1024), (1.0, 2.0), 0.7, 0.2),
]


@pytest.mark.parametrize("shape,L,mu,nu", FLOAT_PAIR_SHAPES)
def test_float_pair_operator_matches_oracle(shape, L, mu, nu):
    import torch
    from bri17_gb300 import wait_timeouts
    h, ho = pair(shape, L, mu, nu)
    rng = np.random.default_rng(21)
    u = mean_free_normal(rng, len(shape), shape)
    ud = to_dev(u)
    f64 = h.apply_stiffness(ud)
    h.set_float_pair(True)
    f_ref = O.apply_stiffness(ho, u)
    for form in ("staged", "tma"):
        h.fused_form = form
        f = h.apply_stiffness(ud)
        torch.cuda.synchronize()
        assert rel_l2(f.cpu().numpy(), f_ref) <= TOL_F64, form
        assert float((f - f64).norm() / f64.norm()) <= 1e-13, form
    assert wait_timeouts() == 0
    for scale in (1e-12, 1e12):
        f = h.apply_stiffness(ud * scale)
        assert rel_l2(f.cpu().numpy(), f_ref * scale) <= TOL_F64, scale
    h.set_float_pair(False)
    assert torch.equal(h.apply_stiffness(ud), f64)


def test_float_pair_conversions_across_the_range():
    """Doubles outside the conversions' fast range (zeros, magnitudes below
    2^-74) take the general integer conversions, the rest the fast ones;
    both kinds sit in one field.  Each component of the float-pair output
    stays within 1e-13 of the FP64 operator's."""
    import torch
    shape = (64, 64, 128)
    h, _ = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    rng = np.random.default_rng(23)
    u = rng.standard_normal((3,) + shape)
    sel = rng.random(u.shape)
    u[sel < 0.05] = 0.0
    u[(sel >= 0.05) & (sel < 0.10)] *= 1e-28           # below 2^-74: general
    u[(sel >= 0.10) & (sel < 0.15)] *= 2.0 ** -70      # just inside the fast range
    u[(sel >= 0.15) & (sel < 0.16)] *= 2.0 ** 40       # large, well inside the range
    ud = to_dev(u)
    f64 = h.apply_stiffness(ud)
    h.set_float_pair(True)
    try:
        f = h.apply_stiffness(ud)
        torch.cuda.synchronize()
    finally:
        h.set_float_pair(False)
    assert bool(torch.isfinite(f).all())
    for k in range(3):
        assert float((f[k] - f64[k]).norm() / f64[k].norm()) <= 1e-13, k


def test_float_pair_host_buffers_and_rejected_grids():
    import torch
    from bri17_gb300._lib import Bri17Error
    shape = (64, 64, 128)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    h.set_float_pair(True)
    rng = np.random.default_rng(22)
    u = mean_free_normal(rng, 3, shape)
    f_ref = O.apply_stiffness(ho, u)
    assert rel_l2(h.apply_stiffness_host(u), f_ref) <= TOL_F64
    up = torch.from_numpy(u).pin_memory()
    assert rel_l2(h.apply_stiffness_host(up).numpy(), f_ref) <= TOL_F64
    for bad in ((48, 64, 128), (64, 64, 64), (32, 64, 128), (64, 64), (1024, 128)):
        hb, _ = pair(bad, (1.0,) * len(bad), 1.0, 0.3)
        with pytest.raises(Bri17Error):
            hb.set_float_pair(True)
    h32, _ = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3, precision="f32")
    with pytest.raises(Bri17Error):
        h32.set_float_pair(True)
