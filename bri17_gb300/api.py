"""Python host API over the C ABI.

``CartesianGrid`` and ``Hooke`` keep the reference's member names and
meanings (include/bri17/bri17.hpp:34-356); ``Hooke`` additionally owns an
operator handle on the GPU and exposes the whole-field operator, the strain
map, the eigenstress right-hand side and the CG solvers on torch CUDA
tensors.  Every numerical method runs in the CUDA library; nothing here
computes on the CPU.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check


def _torch():
    import torch
    return torch


def _stream_ptr(stream=None):
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _fmt(x: float) -> str:
    """std::ostream default formatting of a double (6 significant digits)."""
    return "%g" % x


class CartesianGrid:
    """A periodic Cartesian grid, include/bri17/bri17.hpp:34-159.

    ``shape`` is the number of cells per axis, ``L`` the box size per axis;
    ``size`` = prod(shape) is the number of cells (= nodes)."""

    def __init__(self, shape: Sequence[int], L: Sequence[float]):
        shape = tuple(int(n) for n in shape)
        L = tuple(float(x) for x in L)
        if len(shape) not in (2, 3) or len(L) != len(shape):
            raise ValueError("DIM must be 2 or 3 and len(L) == len(shape)")
        self._shape = shape
        self._L = L
        self._size = int(np.prod(shape))

    dim = property(lambda self: len(self._shape))
    shape = property(lambda self: self._shape)
    L = property(lambda self: self._L)
    size = property(lambda self: self._size)
    num_nodes_per_cell = property(lambda self: 1 << len(self._shape))

    def __repr__(self) -> str:  # CartesianGrid::repr, :61-69
        return ("CartesianGrid<d," + str(self.dim) + ">{shape={"
                + "".join(f"{n}," for n in self._shape) + "},L={"
                + "".join(f"{_fmt(x)}," for x in self._L) + "}}")

    def get_node_at(self, *idx: int) -> int:
        """Row-major node index, include/bri17/bri17.hpp:78-93."""
        if len(idx) != self.dim:
            raise TypeError(f"expected {self.dim} indices")
        out = 0
        for i, n in zip(idx, self._shape):
            out = out * n + int(i)
        return out

    def get_cell_nodes(self, cell: int):
        """Periodic vertex list of a cell, include/bri17/bri17.hpp:127-158
        (order (i,j[,k]) -> 00[0], 0[0]1, ... with the last axis fastest)."""
        cell = int(cell)
        idx = []
        for n in reversed(self._shape):
            idx.append(cell % n)
            cell //= n
        idx = idx[::-1]
        nxt = [0 if i == n - 1 else i + 1 for i, n in zip(idx, self._shape)]
        nodes = []
        for corner in range(self.num_nodes_per_cell):
            sel = [(corner >> (self.dim - 1 - d)) & 1 for d in range(self.dim)]
            nodes.append(self.get_node_at(*[nxt[d] if sel[d] else idx[d]
                                            for d in range(self.dim)]))
        return nodes


class Hooke:
    """Isotropic Hooke material on a periodic grid with its GPU operator.

    Mirrors bri17::Hooke (include/bri17/bri17.hpp:176-356): ``mu``, ``nu``,
    ``grid``, the per-mode functions, plus operator methods on torch CUDA
    tensors.  ``precision`` is "f64" or "f32" (the scalar type of the fields
    the operator methods take)."""

    def __init__(self, mu: float, nu: float, grid: CartesianGrid, precision: str = "f64"):
        self._mu = float(mu)
        self._nu = float(nu)
        self._grid = grid
        self._precision = precision
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        L = _lib.load()
        shape = (ctypes.c_int * grid.dim)(*grid.shape)
        Ls = (ctypes.c_double * grid.dim)(*grid.L)
        h = ctypes.c_void_p()
        check(L.bri17_op_create(grid.dim, shape, Ls, self._mu, self._nu,
                                _lib.F64 if precision == "f64" else _lib.F32,
                                ctypes.byref(h)), "bri17_op_create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().bri17_op_destroy(h)
            except Exception:
                pass
            self._h = None

    mu = property(lambda self: self._mu)
    nu = property(lambda self: self._nu)
    grid = property(lambda self: self._grid)
    precision = property(lambda self: self._precision)
    handle = property(lambda self: self._h)

    def __repr__(self) -> str:  # Hooke::repr, :197-202 (ends with std::endl)
        return (f"Hooke<d,{self._grid.dim}>{{mu={_fmt(self._mu)},nu={_fmt(self._nu)},"
                f"grid={self._grid!r}\n")

    FUSED_FORMS = ("registers", "staged", "tma", "tma_registers")

    @property
    def fused_form(self) -> str:
        """Form of the fused axis-0 pass (diagnostics): "registers",
        "staged", "tma" or "tma_registers"; FP32 handles pick the fastest at
        creation."""
        f = ctypes.c_int()
        check(_lib.load().bri17_op_fused_form(self._h, ctypes.byref(f)), "bri17_op_fused_form")
        return self.FUSED_FORMS[f.value]

    @fused_form.setter
    def fused_form(self, form: str) -> None:
        check(_lib.load().bri17_op_set_fused_form(self._h, self.FUSED_FORMS.index(form)),
              "bri17_op_set_fused_form")

    def set_float_pair(self, enable: bool) -> None:
        """FP64 handles: apply_stiffness / apply_stiffness_host in float-pair
        arithmetic (48-bit significands on the FP32 pipe; about 1e-14 from
        the FP64 operator).  3D power-of-two grids, shape[0], shape[1] in
        64..512 and shape[2] in 128..1024; raises Bri17Error otherwise."""
        check(_lib.load().bri17_op_set_float_pair(self._h, 1 if enable else 0),
              "bri17_op_set_float_pair")

    def set_material(self, mu: float, nu: float) -> None:
        check(_lib.load().bri17_op_set_material(self._h, float(mu), float(nu)),
              "bri17_op_set_material")
        self._mu, self._nu = float(mu), float(nu)

    @property
    def dtype(self):
        torch = _torch()
        return torch.float64 if self._precision == "f64" else torch.float32

    # -- batched per-mode functions (device tensors) ------------------------
    def _k_tensor(self, k):
        torch = _torch()
        k = torch.as_tensor(np.asarray(k) if not torch.is_tensor(k) else k)
        k = k.to(device="cuda", dtype=torch.int32).reshape(-1, self._grid.dim).contiguous()
        return k

    def modal_stiffness_batch(self, k, stream=None):
        """K(k) for a batch of multi-indices: (n, DIM, DIM) complex128 CUDA
        tensor (Hooke::modal_stiffness, include/bri17/bri17.hpp:247-292)."""
        torch = _torch()
        kd = self._k_tensor(k)
        n = kd.shape[0]
        d = self._grid.dim
        out = torch.empty((n, d, d), dtype=torch.complex128, device="cuda")
        check(_lib.load().bri17_modal_stiffness_batch(
            self._h, ctypes.c_void_p(kd.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
            _stream_ptr(stream)), "bri17_modal_stiffness_batch")
        return out

    def modal_strain_displacement_batch(self, k, stream=None):
        """B(k) for a batch: (n, DIM) complex128 CUDA tensor
        (Hooke::modal_strain_displacement, :212-236)."""
        torch = _torch()
        kd = self._k_tensor(k)
        n = kd.shape[0]
        out = torch.empty((n, self._grid.dim), dtype=torch.complex128, device="cuda")
        check(_lib.load().bri17_modal_strain_displacement_batch(
            self._h, ctypes.c_void_p(kd.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
            _stream_ptr(stream)), "bri17_modal_strain_displacement_batch")
        return out

    def modal_eigenstress_to_opposite_strain_batch(self, k, tau, stream=None):
        """-eps_hat(k) of eigenstress Fourier components tau (n, sym) complex
        (Hooke::modal_eigenstress_to_opposite_strain, :308-355)."""
        torch = _torch()
        kd = self._k_tensor(k)
        n = kd.shape[0]
        sym = 3 if self._grid.dim == 2 else 6
        t = torch.as_tensor(tau).to(device="cuda", dtype=torch.complex128)
        t = t.reshape(n, sym).contiguous()
        out = torch.empty((n, sym), dtype=torch.complex128, device="cuda")
        check(_lib.load().bri17_modal_eigenstress_to_opposite_strain_batch(
            self._h, ctypes.c_void_p(kd.data_ptr()), n, ctypes.c_void_p(t.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), _stream_ptr(stream)),
            "bri17_modal_eigenstress_to_opposite_strain_batch")
        return out

    # -- whole-field operators ---------------------------------------------
    def _field(self, x, comps):
        torch = _torch()
        if not torch.is_tensor(x) or not x.is_cuda:
            raise TypeError("expected a CUDA tensor")
        if x.dtype != self.dtype:
            raise TypeError(f"expected dtype {self.dtype}, got {x.dtype}")
        if x.numel() != comps * self._grid.size:
            raise ValueError(f"expected {comps} x {self._grid.size} values, got {x.numel()}")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x

    def apply_stiffness(self, u, out=None, stream=None):
        """f = K u (StiffnessMatrixFactory::compute_Ku,
        tests/test_bri17.cpp:56-107).  u: (DIM, *shape) CUDA tensor."""
        torch = _torch()
        d = self._grid.dim
        u = self._field(u, d)
        f = torch.empty_like(u) if out is None else self._field(out, d)
        check(_lib.load().bri17_apply_stiffness(
            self._h, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(f.data_ptr()),
            _stream_ptr(stream)), "bri17_apply_stiffness")
        return f

    def apply_stiffness_host(self, u):
        """f = K u with host buffers: a numpy array (copied through device
        staging buffers) or a CPU torch tensor; a page-locked tensor
        (``tensor.pin_memory()``) is read in place by the first pass, and f
        comes back page-locked and written in place by the last."""
        n = self._grid.dim * self._grid.size
        try:
            torch = _torch()
        except ImportError:
            torch = None
        if torch is not None and isinstance(u, torch.Tensor):
            if u.is_cuda:
                raise ValueError("apply_stiffness_host takes host buffers")
            u = u.to(self.dtype).contiguous()
            if u.numel() != n:
                raise ValueError("wrong number of values")
            f = torch.empty(u.shape, dtype=u.dtype, pin_memory=u.is_pinned())
            check(_lib.load().bri17_apply_stiffness_host(
                self._h, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                _stream_ptr()), "bri17_apply_stiffness_host")
            return f
        dt = np.float64 if self._precision == "f64" else np.float32
        u = np.ascontiguousarray(u, dtype=dt)
        if u.size != n:
            raise ValueError("wrong number of values")
        f = np.empty_like(u)
        check(_lib.load().bri17_apply_stiffness_host(
            self._h, u.ctypes.data_as(ctypes.c_void_p), f.ctypes.data_as(ctypes.c_void_p),
            _stream_ptr()), "bri17_apply_stiffness_host")
        return f

    def apply_strain(self, u, stream=None):
        """Cell strains (Mandel) of nodal displacements
        (StrainDisplacementMatrixFactory::compute_Bu,
        tests/test_bri17.cpp:194-245).  Returns (sym, *shape)."""
        torch = _torch()
        d = self._grid.dim
        sym = 3 if d == 2 else 6
        u = self._field(u, d)
        eps = torch.empty((sym,) + self._grid.shape, dtype=self.dtype, device=u.device)
        check(_lib.load().bri17_apply_strain(
            self._h, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(eps.data_ptr()),
            _stream_ptr(stream)), "bri17_apply_strain")
        return eps

    def eigenstress_rhs(self, tau, stream=None):
        """Nodal forces b = -|h| B^T tau of a cell-wise Mandel eigenstress
        tau (sym, *shape).  Returns (DIM, *shape)."""
        torch = _torch()
        d = self._grid.dim
        sym = 3 if d == 2 else 6
        tau = self._field(tau, sym)
        b = torch.empty((d,) + self._grid.shape, dtype=self.dtype, device=tau.device)
        check(_lib.load().bri17_eigenstress_rhs(
            self._h, ctypes.c_void_p(tau.data_ptr()), ctypes.c_void_p(b.data_ptr()),
            _stream_ptr(stream)), "bri17_eigenstress_rhs")
        return b

    def eigenstress_to_opposite_strain(self, tau, stream=None):
        """Opposite strain eta = -eps (sym, *shape) of a cell-wise Mandel
        eigenstress tau (sym, *shape): the field form of
        Hooke::modal_eigenstress_to_opposite_strain as python/demo.py applies
        it mode by mode (the direct solution of the eigenstress problem)."""
        torch = _torch()
        d = self._grid.dim
        sym = 3 if d == 2 else 6
        tau = self._field(tau, sym)
        eta = torch.empty((sym,) + self._grid.shape, dtype=self.dtype, device=tau.device)
        check(_lib.load().bri17_eigenstress_to_opposite_strain(
            self._h, ctypes.c_void_p(tau.data_ptr()), ctypes.c_void_p(eta.data_ptr()),
            _stream_ptr(stream)), "bri17_eigenstress_to_opposite_strain")
        return eta

    def sync_status(self, stream=None) -> int:
        """Synchronise `stream` and return the handle's status: 0, or 11 when
        a bounded device wait of its earlier work ran out (that work's
        output is invalid); each failure is reported once."""
        return _lib.load().bri17_op_sync_status(self._h, _stream_ptr(stream))

    def cg_solve(self, b, x0=None, tol: float = 1e-8, max_iterations: int = 100000,
                 mode: str = "plain", raise_on_failure: bool = True, stream=None):
        """Solve K x = b (zero-mean x) by CG.  b: FP64 CUDA tensor (DIM,
        *shape).  mode "plain" (handle precision) or "mixed" (FP32 inner CG,
        FP64 refinement; FP64 handles).  Returns (x, info dict)."""
        torch = _torch()
        d = self._grid.dim
        if not torch.is_tensor(b) or not b.is_cuda or b.dtype != torch.float64:
            raise TypeError("b must be an FP64 CUDA tensor")
        if b.numel() != d * self._grid.size or not b.is_contiguous():
            raise ValueError("b must be a contiguous (DIM, *shape) tensor")
        if x0 is None:
            x = torch.zeros_like(b)
        else:
            if (not torch.is_tensor(x0) or x0.device != b.device
                    or x0.dtype != torch.float64 or x0.numel() != b.numel()):
                raise ValueError("x0 must be an FP64 tensor on b's device with b's size")
            x = x0.clone().reshape(b.shape).contiguous()
        info = _lib.CgInfo()
        rc = _lib.load().bri17_cg_solve(
            self._h, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
            float(tol), int(max_iterations),
            {"plain": _lib.CG_PLAIN, "mixed": _lib.CG_MIXED,
             "mixed_restart": _lib.CG_MIXED_RESTART}[mode], ctypes.byref(info),
            _stream_ptr(stream))
        out = {"iterations": info.iterations, "outer_iterations": info.outer_iterations,
               "rel_residual": info.rel_residual, "status": info.status,
               "status_text": _lib.STATUS.get(info.status, str(info.status))}
        if rc != 0 and raise_on_failure:
            check(rc, "bri17_cg_solve")
        return x, out


def set_wait_limit_ns(ns: int) -> None:
    """Limit (ns of GPU global time) of the first wait on tile copies in the
    tensor-copy kernels on the current device; 0 makes those waits give up
    at once (diagnostics: tests of the failure path).  Default
    1_000_000_000."""
    check(_lib.load().bri17_set_wait_limit_ns(int(ns)), "bri17_set_wait_limit_ns")


def wait_timeouts() -> int:
    """Bounded device waits that ran out on the current device since the
    previous call (0 in normal operation)."""
    n = ctypes.c_int()
    check(_lib.load().bri17_wait_timeouts(ctypes.byref(n)), "bri17_wait_timeouts")
    return n.value


def version() -> str:
    return _lib.load().bri17_version().decode()
