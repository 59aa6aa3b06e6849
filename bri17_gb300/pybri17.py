"""Drop-in for the reference's Python module ``pybri17``
(python/pybri17.cpp:98-107), rebound on the GPU library.

Same classes, members and argument conventions:

* ``CartesianGrid2f64(shape, L)`` / ``CartesianGrid3f64``: static ``dtype``
  and ``dim``; ``shape``, ``size``, ``L``, ``__repr__``, ``get_cell_nodes``,
  ``get_node_at(i, j[, k])`` (python/pybri17.cpp:32-61);
* ``Hooke2f64(mu, nu, grid)`` / ``Hooke3f64``: ``mu``, ``nu``, ``grid``,
  ``__repr__``, and the per-mode methods writing into caller-provided 1-D
  contiguous arrays -- ``modal_strain_displacement(k, B)``,
  ``modal_stiffness_matrix(k, K)``,
  ``modal_eigenstress_to_opposite_strain(k, tau, eta)``
  (python/pybri17.cpp:63-96); a non-contiguous or non-1-D output raises
  ValueError exactly as ``check_contiguous`` does (:9-15);
* module attributes ``__author__`` and ``__version__`` (:100-101).

Beyond the reference, every Hooke class carries the batched and whole-field
methods of :class:`bri17_gb300.api.Hooke` (``modal_stiffness_batch``,
``apply_stiffness``, ``apply_strain``, ``eigenstress_rhs``, ``cg_solve``),
which remove the per-mode Python round trip of python/demo.py:34-40.
The per-mode methods run the same CUDA kernels with a batch of one, through
the host-buffer entry points (bri17_modal_*_host): the caller's numpy arrays
are staged in page-locked memory the handle keeps, one kernel runs, and the
result is written into the caller's array -- no device allocation or torch
round trip per call.

``import pybri17`` (the reference's module name) finds this module through
the top-level ``pybri17.py`` beside this package.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, api
from ._lib import check

__author__ = "S. Brisard"
__version__ = "0.1"


def _check_contiguous(a, dtype):
    """python/pybri17.cpp:9-15: one-dimensional and contiguous, else
    ValueError (std::invalid_argument maps to ValueError in pybind11).  An
    array of another dtype raises TypeError: the reference's py::array_t
    would convert it to a temporary copy and write there."""
    if isinstance(a, np.ndarray) and a.dtype != dtype:
        raise TypeError(f"expected dtype {np.dtype(dtype)}, got {a.dtype}")
    if not isinstance(a, np.ndarray) or a.ndim != 1 or a.strides[0] != np.dtype(dtype).itemsize:
        raise ValueError("expected one-dimensional, contiguous array")


class _GridBase(api.CartesianGrid):
    dtype = np.dtype(np.float64)
    _DIM = 0

    def __init__(self, shape, L):
        if len(shape) != self._DIM or len(L) != self._DIM:
            raise TypeError(f"expected {self._DIM} values for shape and L")
        super().__init__(shape, L)

    def get_cell_nodes(self, cell):
        return list(super().get_cell_nodes(cell))


class CartesianGrid2f64(_GridBase):
    _DIM = 2
    dim = 2

    def get_node_at(self, i, j):
        return super().get_node_at(i, j)


class CartesianGrid3f64(_GridBase):
    _DIM = 3
    dim = 3

    def get_node_at(self, i, j, k):
        return super().get_node_at(i, j, k)


class _HookeBase(api.Hooke):
    _DIM = 0
    _GRID = None

    def __init__(self, mu, nu, grid):
        if not isinstance(grid, _GridBase) or grid.dim != self._DIM:
            raise TypeError(f"expected a CartesianGrid{self._DIM}f64")
        # The reference copies the grid (include/bri17/bri17.hpp:193-194).
        super().__init__(mu, nu, type(grid)(grid.shape, grid.L), precision="f64")

    def _k(self, k):
        k = np.asarray(k, dtype=np.intc)
        _check_contiguous(k, np.intc)
        if k.shape[0] < self._DIM:
            raise ValueError(f"expected {self._DIM} frequency indices")
        return k

    @staticmethod
    def _room(a, n):
        if a.shape[0] < n:
            raise ValueError(f"expected an array of at least {n} entries")

    def modal_strain_displacement(self, k, B):
        _check_contiguous(B, np.complex128)
        k = self._k(k)
        self._room(B, self._DIM)
        check(_lib.load().bri17_modal_strain_displacement_host(
            self.handle, k.ctypes.data_as(ctypes.c_void_p), 1,
            B.ctypes.data_as(ctypes.c_void_p)), "bri17_modal_strain_displacement_host")

    def modal_stiffness_matrix(self, k, K):
        _check_contiguous(K, np.complex128)
        k = self._k(k)
        self._room(K, self._DIM * self._DIM)
        check(_lib.load().bri17_modal_stiffness_host(
            self.handle, k.ctypes.data_as(ctypes.c_void_p), 1,
            K.ctypes.data_as(ctypes.c_void_p)), "bri17_modal_stiffness_host")

    def modal_eigenstress_to_opposite_strain(self, k, tau, eta):
        _check_contiguous(tau, np.complex128)
        _check_contiguous(eta, np.complex128)
        sym = 3 if self._DIM == 2 else 6
        # The reference does not check k here (python/pybri17.cpp:91-92); it
        # is read as DIM int32 values.
        k = np.ascontiguousarray(np.asarray(k, dtype=np.intc).reshape(-1)[: self._DIM])
        if k.shape[0] < self._DIM:
            raise ValueError(f"expected {self._DIM} frequency indices")
        self._room(tau, sym)
        self._room(eta, sym)
        check(_lib.load().bri17_modal_eigenstress_to_opposite_strain_host(
            self.handle, k.ctypes.data_as(ctypes.c_void_p), 1,
            tau.ctypes.data_as(ctypes.c_void_p), eta.ctypes.data_as(ctypes.c_void_p)),
            "bri17_modal_eigenstress_to_opposite_strain_host")


class Hooke2f64(_HookeBase):
    _DIM = 2


class Hooke3f64(_HookeBase):
    _DIM = 3
