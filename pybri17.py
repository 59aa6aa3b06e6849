"""``import pybri17``: the reference's Python module name
(python/pybri17.cpp:98, ``PYBIND11_MODULE(pybri17, m)``), served by the GPU
library.  Everything is defined in :mod:`bri17_gb300.pybri17`; this module
re-exports it under the reference's name so that code written against the
reference imports it unchanged."""
from bri17_gb300.pybri17 import (  # noqa: F401
    CartesianGrid2f64,
    CartesianGrid3f64,
    Hooke2f64,
    Hooke3f64,
    __author__,
    __version__,
)
