"""bri17_gb300: GB300 (sm_103a) implementation of the bri17 matrix-free
periodic finite-element stiffness operator, with CG solvers and a
continuous-batching solve server.

The compute path is the CUDA library ``libbri17_gb300.so`` (C ABI in
``include/bri17_gb300.h``); this package binds it.  ``pybri17`` re-exports
the reference's Python module surface on top of it.
"""
from .api import CartesianGrid, Hooke, set_wait_limit_ns, version, wait_timeouts  # noqa: F401

__version__ = "0.1.0"
