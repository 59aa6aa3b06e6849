"""CPU oracle for the bri17 periodic stiffness operator.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; it is the checker of the
GPU library, never part of it.

The per-mode arithmetic lives in ``oracle/bri17_oracle.c`` (a line-by-line
restatement of ``include/bri17/bri17.hpp`` of sbrisard/bri17).  This module
restates the reference's operator application, which lives only in its test
harness, with numpy's pocketfft standing in for FFTW3 (the reference links
FFTW3 with an unpinned version, tests/CMakeLists.txt:15-17):

* ``apply_stiffness``: ``StiffnessMatrixFactory::compute_Ku``,
  tests/test_bri17.cpp:56-107 -- DIM complex-to-complex forward DFTs, the
  per-mode K(k) u(k) loop, DIM unnormalised backward DFTs, then the factor
  ``|h| / |N|``.
* ``apply_strain``: ``StrainDisplacementMatrixFactory::compute_Bu``,
  tests/test_bri17.cpp:194-245, factor ``1 / |N|``.
* ``stiffness_matrix`` / ``strain_displacement_matrix``: the dense-matrix
  extraction by unit vectors of tests/test_bri17.cpp:130-150 and :271-292,
  with the ``|imag| <= 1e-14`` check of :140-144.
* ``assemble_stiffness`` / ``assemble_strain_displacement``: the real-space
  assembly of element matrices, tests/test_bri17.cpp:153-174 and :295-316.
* ``eigenstress_rhs`` / ``eigenstress_solve``: the periodic eigenstress
  problem whose per-mode solve is include/bri17/bri17.hpp:308-355.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbri17_oracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libbri17_ref.so")
_lock = threading.Lock()
_lib = None
_ref = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(quiet: bool = True) -> None:
    """Compile the C restatement (and, where the reference checkout is
    present, the reference header) with ``make -C oracle``."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", _HERE, "all"], check=True, stdout=out)
    subprocess.run(["make", "-C", _HERE, "ref-if-present"], check=True, stdout=out)


def ref_root() -> str:
    """Where oracle/Makefile reads the reference checkout (BRI17_REF_ROOT
    overrides its default)."""
    r = subprocess.run(["make", "-s", "-C", _HERE, "print-ref-root"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.isfile(_LIB_PATH):
                build()
            L = ctypes.CDLL(_LIB_PATH)
            common = [ctypes.c_int, _ip, _dp, ctypes.c_double, ctypes.c_double]
            for name in ("oracle_modal_stiffness", "oracle_modal_strain_displacement"):
                getattr(L, name).argtypes = common + [_ip, _dp]
            L.oracle_modal_eigenstress_to_opposite_strain.argtypes = common + [_ip, _dp, _dp]
            for name in ("oracle_modal_stiffness_batch",
                         "oracle_modal_strain_displacement_batch"):
                getattr(L, name).argtypes = common + [_ip, ctypes.c_int64, _dp]
            for name in ("oracle_stiffness_modal_apply", "oracle_strain_modal_apply",
                         "oracle_eigenstress_modal_solve", "oracle_eigenstress_modal_rhs",
                         "oracle_eigenstress_modal_eta", "oracle_eigenstress_modal_solve_half"):
                getattr(L, name).argtypes = common + [_dp, _dp]
            L.oracle_get_cell_nodes.argtypes = [ctypes.c_int, _ip, ctypes.c_int, _ip]
            L.oracle_get_node_at.argtypes = [ctypes.c_int, _ip, _ip]
            L.oracle_get_node_at.restype = ctypes.c_int
            L.oracle_num_threads.restype = ctypes.c_int
            L.oracle_set_num_threads.argtypes = [ctypes.c_int]
            _lib = L
    return _lib


def ref_lib():
    """The reference's own header compiled into oracle/_ref, or None."""
    global _ref
    with _lock:
        if _ref is None and os.path.isfile(_REF_PATH):
            R = ctypes.CDLL(_REF_PATH)
            common = [ctypes.c_int, _ip, _dp, ctypes.c_double, ctypes.c_double]
            R.ref_modal_stiffness_batch.argtypes = common + [_ip, ctypes.c_long, _dp]
            R.ref_modal_strain_displacement_batch.argtypes = common + [_ip, ctypes.c_long, _dp]
            R.ref_all_cell_nodes.argtypes = [ctypes.c_int, _ip, _ip]
            R.ref_repr.argtypes = common + [ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
            R.ref_repr.restype = ctypes.c_int
            _ref = R
    return _ref


def _iarr(x):
    a = np.ascontiguousarray(x, dtype=np.intc)
    return a, a.ctypes.data_as(_ip)


def _darr(x):
    a = np.ascontiguousarray(x, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


class Grid:
    """Shape, box size and derived quantities of a CartesianGrid
    (include/bri17/bri17.hpp:34-58)."""

    def __init__(self, shape, L):
        self.shape = tuple(int(n) for n in shape)
        self.L = tuple(float(x) for x in L)
        self.dim = len(self.shape)
        if self.dim not in (2, 3) or len(self.L) != self.dim:
            raise ValueError("DIM must be 2 or 3")
        self.size = int(np.prod(self.shape))
        self.h = tuple(L_ / n for L_, n in zip(self.L, self.shape))
        cv = 1.0
        for i in range(self.dim):
            cv *= self.L[i] / self.shape[i]
        self.cell_volume = cv  # accumulated like tests/test_bri17.cpp:93-97


class Hooke:
    """Material + grid, as in include/bri17/bri17.hpp:176-194."""

    def __init__(self, mu, nu, grid: Grid):
        self.mu = float(mu)
        self.nu = float(nu)
        self.grid = grid

    def _common(self):
        g = self.grid
        shape, sp = _iarr(g.shape)
        L, Lp = _darr(g.L)
        return (g.dim, sp, Lp, self.mu, self.nu), (shape, L)

    # -- per-mode functions -------------------------------------------------
    def modal_stiffness(self, k):
        """K(k) as complex128 (n, DIM, DIM) for k of shape (n, DIM) or (DIM,)."""
        k = np.asarray(k, dtype=np.intc)
        single = k.ndim == 1
        k = np.atleast_2d(k)
        n, dim = k.shape
        out = np.empty((n, dim * dim), dtype=np.complex128)
        args, keep = self._common()
        ka, kp = _iarr(k)
        lib().oracle_modal_stiffness_batch(*args, kp, n, out.ctypes.data_as(_dp))
        out = out.reshape(n, dim, dim)
        return out[0] if single else out

    def modal_strain_displacement(self, k):
        k = np.asarray(k, dtype=np.intc)
        single = k.ndim == 1
        k = np.atleast_2d(k)
        n, dim = k.shape
        out = np.empty((n, dim), dtype=np.complex128)
        args, keep = self._common()
        ka, kp = _iarr(k)
        lib().oracle_modal_strain_displacement_batch(*args, kp, n, out.ctypes.data_as(_dp))
        return out[0] if single else out

    def modal_eigenstress_to_opposite_strain(self, k, tau):
        dim = self.grid.dim
        sym = 3 if dim == 2 else 6
        eta = np.empty(sym, dtype=np.complex128)
        tau = np.ascontiguousarray(tau, dtype=np.complex128)
        args, keep = self._common()
        ka, kp = _iarr(k)
        lib().oracle_modal_eigenstress_to_opposite_strain(
            *args, kp, tau.ctypes.data_as(_dp), eta.ctypes.data_as(_dp))
        return eta

    # -- whole-field modal loops ------------------------------------------
    def _modal_loop(self, fn, xhat, ncomp_out):
        g = self.grid
        xhat = np.ascontiguousarray(xhat, dtype=np.complex128)
        out = np.empty((ncomp_out,) + g.shape, dtype=np.complex128)
        args, keep = self._common()
        fn(*args, xhat.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
        return out


def _axes(dim):
    return tuple(range(1, dim + 1))


def apply_stiffness(hooke: Hooke, u, return_complex=False):
    """f = K u, restating compute_Ku (tests/test_bri17.cpp:56-107).

    ``u`` has shape (DIM, *grid.shape) (SoA, row-major nodes)."""
    g = hooke.grid
    u = np.asarray(u, dtype=np.float64).reshape((g.dim,) + g.shape)
    uhat = np.fft.fftn(u.astype(np.complex128), axes=_axes(g.dim))
    Kuhat = hooke._modal_loop(lib().oracle_stiffness_modal_apply, uhat, g.dim)
    Ku = np.fft.ifftn(Kuhat, axes=_axes(g.dim), norm="forward")  # FFTW_BACKWARD
    Ku *= g.cell_volume / g.size
    return Ku if return_complex else Ku.real.copy()


def apply_strain(hooke: Hooke, u, return_complex=False):
    """Cell strains (Mandel) of nodal displacements u, restating compute_Bu
    (tests/test_bri17.cpp:194-245)."""
    g = hooke.grid
    sym = 3 if g.dim == 2 else 6
    u = np.asarray(u, dtype=np.float64).reshape((g.dim,) + g.shape)
    uhat = np.fft.fftn(u.astype(np.complex128), axes=_axes(g.dim))
    ehat = hooke._modal_loop(lib().oracle_strain_modal_apply, uhat, sym)
    e = np.fft.ifftn(ehat, axes=_axes(g.dim), norm="forward")
    e *= 1.0 / g.size
    return e if return_complex else e.real.copy()


def stiffness_matrix(hooke: Hooke, imag_tol=1e-14):
    """Dense global K by unit-vector probing, tests/test_bri17.cpp:130-150."""
    g = hooke.grid
    n = g.dim * g.size
    K = np.empty((n, n))
    u = np.zeros(n)
    for j in range(n):
        u[j] = 1.0
        col = apply_stiffness(hooke, u, return_complex=True).reshape(n)
        if np.max(np.abs(col.imag)) > imag_tol:
            raise RuntimeError(f"imag(K[:, {j}]) exceeds {imag_tol}")
        K[:, j] = col.real
        u[j] = 0.0
    return K


def strain_displacement_matrix(hooke: Hooke, imag_tol=1e-14):
    """Dense global B by unit-vector probing, tests/test_bri17.cpp:271-292."""
    g = hooke.grid
    sym = 3 if g.dim == 2 else 6
    n = g.dim * g.size
    B = np.empty((sym * g.size, n))
    u = np.zeros(n)
    for j in range(n):
        u[j] = 1.0
        col = apply_strain(hooke, u, return_complex=True).reshape(-1)
        if np.max(np.abs(col.imag)) > imag_tol:
            raise RuntimeError(f"imag(B[:, {j}]) exceeds {imag_tol}")
        B[:, j] = col.real
        u[j] = 0.0
    return B


def cell_nodes(grid: Grid):
    """All cells' vertex lists, include/bri17/bri17.hpp:127-158."""
    shape, sp = _iarr(grid.shape)
    nn = 1 << grid.dim
    out = np.empty((grid.size, nn), dtype=np.intc)
    tmp = np.empty(nn, dtype=np.intc)
    for c in range(grid.size):
        lib().oracle_get_cell_nodes(grid.dim, sp, c, tmp.ctypes.data_as(_ip))
        out[c] = tmp
    return out


def assemble_stiffness(grid: Grid, Ke):
    """Real-space assembly, tests/test_bri17.cpp:153-174."""
    nn = 1 << grid.dim
    n = grid.dim * grid.size
    K = np.zeros((n, n))
    nodes = cell_nodes(grid)
    for cell in range(grid.size):
        idx = [nodes[cell][ie % nn] + grid.size * (ie // nn) for ie in range(nn * grid.dim)]
        for a, i in enumerate(idx):
            for b, j in enumerate(idx):
                K[i, j] += Ke[a, b]
    return K


def assemble_strain_displacement(grid: Grid, Be):
    """Real-space assembly, tests/test_bri17.cpp:295-316."""
    nn = 1 << grid.dim
    sym = 3 if grid.dim == 2 else 6
    B = np.zeros((sym * grid.size, grid.dim * grid.size))
    nodes = cell_nodes(grid)
    for cell in range(grid.size):
        for il in range(sym):
            i = il * grid.size + cell
            for jl in range(nn * grid.dim):
                j = nodes[cell][jl % nn] + grid.size * (jl // nn)
                B[i, j] += Be[il, jl]
    return B


def eigenstress_rhs(hooke: Hooke, tau):
    """Nodal forces b of a cell-wise eigenstress tau (Mandel, (sym, *shape)):
    b = -|h| ifft(tau_hat . conj(B)), so that K u = b is the equilibrium
    problem of sphinx/theory.rst eq. (15)-(17) whose per-mode system is
    include/bri17/bri17.hpp:340-341 (solved there for -u)."""
    g = hooke.grid
    tau = np.asarray(tau, dtype=np.float64).reshape((-1,) + g.shape)
    tauhat = np.fft.fftn(tau.astype(np.complex128), axes=_axes(g.dim))
    bhat = hooke._modal_loop(lib().oracle_eigenstress_modal_rhs, tauhat, g.dim)
    b = np.fft.ifftn(bhat, axes=_axes(g.dim))
    return -(g.cell_volume * b.real)


def eigenstress_solve(hooke: Hooke, tau):
    """Exact mean-free solution u of K u = eigenstress_rhs(tau) by the
    per-mode direct solve of include/bri17/bri17.hpp:308-341 (k = 0 -> 0)."""
    g = hooke.grid
    tau = np.asarray(tau, dtype=np.float64).reshape((-1,) + g.shape)
    tauhat = np.fft.fftn(tau.astype(np.complex128), axes=_axes(g.dim))
    uhat = hooke._modal_loop(lib().oracle_eigenstress_modal_solve, tauhat, g.dim)
    return -np.fft.ifftn(uhat, axes=_axes(g.dim)).real


def eigenstress_solve_half(hooke: Hooke, tau, workers: int = 1):
    """The solution of ``eigenstress_solve`` through real-to-complex DFTs:
    only the half spectrum k_last in [0, N_last/2] is transformed and solved
    (oracle_eigenstress_modal_solve_half, every kept mode as in
    include/bri17/bri17.hpp:308-341), and the inverse real DFT restores the
    conjugate half.  Same result to rounding, with half the transform work
    and ``workers`` FFT threads (scipy.fft where present), so that it runs at
    the large grids of the solver measurements."""
    g = hooke.grid
    tau = np.asarray(tau, dtype=np.float64).reshape((-1,) + g.shape)
    axes = _axes(g.dim)
    try:
        import scipy.fft as sf

        def rfftn(a):
            return sf.rfftn(a, axes=axes, workers=workers)

        def irfftn(a):
            return sf.irfftn(a, s=g.shape, axes=axes, workers=workers)
    except ImportError:  # numpy's pocketfft, one thread
        def rfftn(a):
            return np.fft.rfftn(a, axes=axes)

        def irfftn(a):
            return np.fft.irfftn(a, s=g.shape, axes=axes)
    tauhat = np.ascontiguousarray(rfftn(tau), dtype=np.complex128)
    del tau
    hshape = g.shape[:-1] + (g.shape[-1] // 2 + 1,)
    uhat = np.empty((g.dim,) + hshape, dtype=np.complex128)
    args, keep = hooke._common()
    lib().oracle_eigenstress_modal_solve_half(*args, tauhat.ctypes.data_as(_dp),
                                              uhat.ctypes.data_as(_dp))
    del tauhat
    return -irfftn(uhat)


def eigenstress_opposite_strain(hooke: Hooke, tau):
    """Opposite strain field eta = ifft(eta_hat(fft(tau))) with eta_hat the
    per-mode Hooke::modal_eigenstress_to_opposite_strain
    (include/bri17/bri17.hpp:308-355) over every mode, as python/demo.py:24-40
    runs it; (sym, *shape) real."""
    g = hooke.grid
    sym = 3 if g.dim == 2 else 6
    tau = np.asarray(tau, dtype=np.float64).reshape((sym,) + g.shape)
    tauhat = np.fft.fftn(tau.astype(np.complex128), axes=_axes(g.dim))
    etahat = hooke._modal_loop(lib().oracle_eigenstress_modal_eta, tauhat, sym)
    return np.fft.ifftn(etahat, axes=_axes(g.dim)).real


def set_num_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())
