"""Pins the CPU oracle (oracle/) to the reference.

* The reference's own golden test (tests/test_bri17.cpp:318-606): dense K and
  B extracted from the operator by unit vectors must equal the real-space
  assembly of the Maxima element matrices, |a - e| <= 1e-15 |e| + 1e-14, and
  every extracted entry must be real to 1e-14.
* The per-mode functions against outputs of the reference header itself
  (tests/golden/modal_ref.npz, written by tests/golden/make_golden.py from
  include/bri17/bri17.hpp compiled unmodified): bit for bit.
* Where oracle/_ref is present (the container that has the reference), the
  same comparison live on further grids, and the repr strings.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _assert_close(expected, actual, rtol, atol):
    err = np.abs(actual - expected)
    tol = rtol * np.abs(expected) + atol
    bad = np.argwhere(err > tol)
    assert bad.size == 0, f"{len(bad)} entries off, first {bad[0]}: {expected[tuple(bad[0])]} vs {actual[tuple(bad[0])]}"


@pytest.mark.parametrize("case_index", [0, 1, 2, 3])
def test_golden_element_matrices(golden_elements, case_index):
    g = golden_elements
    case = g["cases"][case_index]
    grid = O.Grid(case["shape"], case["L"])
    hooke = O.Hooke(g["mu"], g["nu"], grid)
    E = np.array(case["values"]).reshape(case["rows"], case["cols"])
    if case["kind"] == "K":
        expected = O.assemble_stiffness(grid, E)
        actual = O.stiffness_matrix(hooke, imag_tol=g["imag_tol"])
    else:
        expected = O.assemble_strain_displacement(grid, E)
        actual = O.strain_displacement_matrix(hooke, imag_tol=g["imag_tol"])
    _assert_close(expected, actual, g["rtol"], g["atol"])


def test_golden_detects_a_planted_error(golden_elements):
    """The comparison fails when the oracle's operator is perturbed by one
    part in 1e12 (the check is live, not vacuous)."""
    g = golden_elements
    case = g["cases"][1]
    grid = O.Grid(case["shape"], case["L"])
    hooke = O.Hooke(g["mu"] * (1 + 1e-12), g["nu"], grid)
    E = np.array(case["values"]).reshape(case["rows"], case["cols"])
    with pytest.raises(AssertionError):
        _assert_close(O.assemble_stiffness(grid, E), O.stiffness_matrix(hooke),
                      g["rtol"], g["atol"])


def test_modal_functions_bit_exact_vs_reference_fixture(golden_modal):
    for c in golden_modal:
        grid = O.Grid(c["shape"], c["L"])
        h = O.Hooke(c["mu"], c["nu"], grid)
        K = h.modal_stiffness(c["k"]).reshape(c["K"].shape)
        B = h.modal_strain_displacement(c["k"])
        assert np.array_equal(K.view(np.float64), c["K"].view(np.float64)), c["shape"]
        assert np.array_equal(B.view(np.float64), c["B"].view(np.float64)), c["shape"]


def test_cell_nodes_vs_reference_fixture(golden_modal):
    for c in golden_modal:
        grid = O.Grid(c["shape"], c["L"])
        assert np.array_equal(O.cell_nodes(grid), c["nodes"])


def test_modal_stiffness_symmetry_and_null_mode(golden_modal):
    for c in golden_modal:
        grid = O.Grid(c["shape"], c["L"])
        h = O.Hooke(c["mu"], c["nu"], grid)
        K = h.modal_stiffness(c["k"])
        assert np.all(K.imag == 0)
        assert np.array_equal(K, np.swapaxes(K, 1, 2))
        K0 = h.modal_stiffness(np.zeros(grid.dim, dtype=np.intc))
        assert np.all(K0 == 0)


def test_eigenstress_solution_satisfies_equilibrium():
    """u = eigenstress_solve(tau) solves K u = eigenstress_rhs(tau) with the
    operator restated from compute_Ku, and is mean-free."""
    rng = np.random.default_rng(5)
    for shape, L in (((6, 5), (1.0, 1.3)), ((4, 6, 5), (1.0, 0.7, 1.2))):
        grid = O.Grid(shape, L)
        h = O.Hooke(1.3, 0.27, grid)
        sym = 3 if grid.dim == 2 else 6
        tau = rng.standard_normal((sym,) + shape)
        b = O.eigenstress_rhs(h, tau)
        u = O.eigenstress_solve(h, tau)
        Ku = O.apply_stiffness(h, u)
        assert np.abs(Ku - b).max() <= 1e-12 * np.abs(b).max()
        assert np.abs(u.reshape(grid.dim, -1).mean(axis=1)).max() < 1e-13 * np.abs(u).max()


def test_eigenstress_rhs_matches_real_space_assembly(golden_elements):
    """b = -|h| B^T tau with B the golden real-space strain-displacement
    matrix (Maxima Be, tests/test_bri17.cpp:547-552, :570-598)."""
    g = golden_elements
    rng = np.random.default_rng(9)
    for case in g["cases"][2:]:
        grid = O.Grid(case["shape"], case["L"])
        h = O.Hooke(g["mu"], g["nu"], grid)
        Bmat = O.assemble_strain_displacement(
            grid, np.array(case["values"]).reshape(case["rows"], case["cols"]))
        sym = 3 if grid.dim == 2 else 6
        tau = rng.standard_normal(sym * grid.size)
        b = O.eigenstress_rhs(h, tau.reshape((sym,) + grid.shape)).reshape(-1)
        assert np.allclose(b, -grid.cell_volume * Bmat.T @ tau, rtol=0, atol=1e-13)


def test_modal_eigenstress_per_mode_matches_field_solve():
    """The per-mode opposite strain (include/bri17/bri17.hpp:308-355) equals
    minus the DFT of the strain of the field solution."""
    rng = np.random.default_rng(11)
    grid = O.Grid((4, 5, 6), (1.0, 1.1, 0.9))
    h = O.Hooke(2.0, 0.3, grid)
    tau = rng.standard_normal((6,) + grid.shape)
    u = O.eigenstress_solve(h, tau)
    eps = O.apply_strain(h, u)
    eps_hat = np.fft.fftn(eps, axes=(1, 2, 3))
    tau_hat = np.fft.fftn(tau, axes=(1, 2, 3))
    for k in ((0, 0, 0), (1, 2, 3), (3, 4, 5), (2, 0, 1)):
        eta = h.modal_eigenstress_to_opposite_strain(np.array(k, dtype=np.intc),
                                                     tau_hat[(slice(None),) + k])
        assert np.allclose(eta, -eps_hat[(slice(None),) + k], rtol=1e-12, atol=1e-12)


ref = O.ref_lib()


@pytest.mark.skipif(ref is None, reason="oracle/_ref not built (needs the reference checkout)")
def test_oracle_bit_exact_vs_live_reference():
    rng = np.random.default_rng(3)
    for trial in range(12):
        dim = 2 + trial % 2
        shape = tuple(int(n) for n in rng.integers(1, 40, size=dim))
        L = tuple(float(x) for x in rng.uniform(0.1, 10.0, size=dim))
        mu, nu = float(rng.uniform(0.1, 10)), float(rng.uniform(-0.9, 0.49))
        k = rng.integers(-100, 100, size=(500, dim)).astype(np.intc)
        grid = O.Grid(shape, L)
        h = O.Hooke(mu, nu, grid)
        sa, sp = O._iarr(shape)
        La, Lp = O._darr(L)
        K = np.empty((500, dim * dim), dtype=np.complex128)
        B = np.empty((500, dim), dtype=np.complex128)
        ref.ref_modal_stiffness_batch(dim, sp, Lp, mu, nu, k.ctypes.data_as(O._ip), 500,
                                      K.ctypes.data_as(O._dp))
        ref.ref_modal_strain_displacement_batch(dim, sp, Lp, mu, nu, k.ctypes.data_as(O._ip),
                                                500, B.ctypes.data_as(O._dp))
        assert np.array_equal(h.modal_stiffness(k).reshape(500, -1).view(np.float64),
                              K.view(np.float64))
        assert np.array_equal(h.modal_strain_displacement(k).view(np.float64),
                              B.view(np.float64))


@pytest.mark.skipif(ref is None, reason="oracle/_ref not built (needs the reference checkout)")
def test_repr_strings_match_reference():
    import ctypes

    from bri17_gb300.api import CartesianGrid, _fmt
    for shape, L, mu, nu in (((3, 4), (3.3000000000000003, 4.8), 5.6, 0.3),
                             ((3, 4, 5), (1.0, 0.125, 12.5), 1.0, 0.25)):
        dim = len(shape)
        sa, sp = O._iarr(shape)
        La, Lp = O._darr(L)
        buf = ctypes.create_string_buffer(512)
        ref.ref_repr(dim, sp, Lp, mu, nu, 0, buf, 512)
        assert repr(CartesianGrid(shape, L)) == buf.value.decode()
        ref.ref_repr(dim, sp, Lp, mu, nu, 1, buf, 512)
        expected = (f"Hooke<d,{dim}>{{mu={_fmt(mu)},nu={_fmt(nu)},grid="
                    f"{CartesianGrid(shape, L)!r}\n")
        assert expected == buf.value.decode()


def test_opposite_strain_field_restatement():
    """The field form of modal_eigenstress_to_opposite_strain agrees with the
    per-mode restatement at a mode, and eta = -eps(u) for the direct
    displacement solve u of the same eigenstress (include/bri17/bri17.hpp:300,
    :342: the reference's modal u is the negative displacement)."""
    g = O.Grid((6, 5, 4), (1.0, 1.2, 0.8))
    h = O.Hooke(1.3, 0.3, g)
    rng = np.random.default_rng(0)
    tau = rng.standard_normal((6, 6, 5, 4))
    eta = O.eigenstress_opposite_strain(h, tau)
    tauhat = np.fft.fftn(tau.astype(complex), axes=(1, 2, 3))
    etahat = np.fft.fftn(eta.astype(complex), axes=(1, 2, 3))
    for k in ((2, 1, 3), (0, 0, 1), (5, 4, 2)):
        e = h.modal_eigenstress_to_opposite_strain(np.array(k, dtype=np.intc),
                                                   tauhat[(slice(None),) + k].copy())
        assert np.abs(e - etahat[(slice(None),) + k]).max() <= 1e-13 * np.abs(etahat).max()
    assert np.abs(etahat[:, 0, 0, 0]).max() <= 1e-13 * np.abs(etahat).max()
    eps = O.apply_strain(h, O.eigenstress_solve(h, tau))
    assert np.abs(eta + eps).max() <= 1e-13 * np.abs(eta).max()


def _make_golden():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.skipif(not __import__("os").path.isdir(_make_golden().default_ref_root()),
                    reason="needs the reference checkout")
def test_golden_fixtures_regenerate_identically(tmp_path):
    """tests/golden/make_golden.py, run again on the reference, writes the
    committed fixtures: the same JSON text and bit-identical arrays."""
    import os
    mg = _make_golden()
    mg.main(["--out-dir", str(tmp_path)])
    here = os.path.join(os.path.dirname(__file__), "golden")
    for name in ("element_matrices.json", "modal_ref.json"):
        with open(os.path.join(here, name)) as a, open(tmp_path / name) as b:
            assert a.read() == b.read(), name
    a = np.load(os.path.join(here, "modal_ref.npz"))
    b = np.load(tmp_path / "modal_ref.npz")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert a[k].dtype == b[k].dtype and np.array_equal(a[k].view(np.uint8),
                                                           b[k].view(np.uint8)), k


def test_oracle_results_do_not_depend_on_thread_count():
    """The per-mode loops split modes across OpenMP threads; every mode is
    independent, so the operator's output is bit-identical for 1 and 4
    threads (the CPU baselines time both)."""
    rng = np.random.default_rng(21)
    grid = O.Grid((12, 10, 9), (1.0, 0.8, 1.1))
    h = O.Hooke(1.0, 0.3, grid)
    u = rng.standard_normal((3,) + grid.shape)
    before = O.num_threads()
    try:
        O.set_num_threads(1)
        f1 = O.apply_stiffness(h, u)
        O.set_num_threads(4)
        f4 = O.apply_stiffness(h, u)
    finally:
        O.set_num_threads(before)
    assert np.array_equal(f1.view(np.uint8), f4.view(np.uint8))


DEGENERATE = [(0, (2, 2)), (0, (1, 5)), (0, (2, 3)), (0, (1, 1)),
              (1, (2, 2, 2)), (1, (1, 3, 2)), (1, (2, 1, 4)), (1, (1, 1, 3)),
              (2, (2, 2)), (2, (1, 5)), (3, (2, 2, 2)), (3, (1, 3, 2))]


@pytest.mark.parametrize("case_index,shape", DEGENERATE)
def test_golden_element_matrices_on_degenerate_grids(golden_elements, case_index, shape):
    """The Maxima element matrices depend only on the cell spacing, so the
    reference's golden check (tests/test_bri17.cpp:318-606) extends to other
    grids of the same spacing: axes of one and two cells, where a cell's
    periodic vertices coincide (include/bri17/bri17.hpp:127-158), at the
    reference's tolerance."""
    g = golden_elements
    case = g["cases"][case_index]
    spacing = [L / n for L, n in zip(case["L"], case["shape"])]
    grid = O.Grid(shape, [n * s for n, s in zip(shape, spacing)])
    hooke = O.Hooke(g["mu"], g["nu"], grid)
    E = np.array(case["values"]).reshape(case["rows"], case["cols"])
    if case["kind"] == "K":
        expected = O.assemble_stiffness(grid, E)
        actual = O.stiffness_matrix(hooke, imag_tol=g["imag_tol"])
    else:
        expected = O.assemble_strain_displacement(grid, E)
        actual = O.strain_displacement_matrix(hooke, imag_tol=g["imag_tol"])
    _assert_close(expected, actual, g["rtol"], g["atol"])


@pytest.mark.parametrize("shape,L", [((6, 5), (1.0, 1.3)), ((8, 7, 5), (1.0, 0.9, 1.2)),
                                     ((7, 9, 6), (1.0, 1.0, 1.0)),
                                     ((16, 1, 12), (1.0, 1.0, 0.5))])
def test_half_spectrum_solve_matches_full_spectrum_solve(shape, L):
    """The half-spectrum form of the modal direct solve (real DFTs, used at
    the solver benchmarks' grid sizes) gives the full-spectrum oracle's
    solution to rounding, on odd, even and one-cell axes."""
    h = O.Hooke(1.3, 0.3, O.Grid(shape, L))
    sym = 3 if len(shape) == 2 else 6
    tau = np.random.default_rng(5).standard_normal((sym,) + shape)
    a = O.eigenstress_solve(h, tau)
    b = O.eigenstress_solve_half(h, tau, workers=2)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)
