"""ctypes binding of ``libbri17_gb300.so`` (C ABI: include/bri17_gb300.h).

Loading fails loudly: there is no CPU fallback for anything this library
computes.  Build the library with ``python bri17_gb300/build.py`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbri17_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "bri17_gb300.h")

_lib = None

c_int_p = ctypes.POINTER(ctypes.c_int)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
vp = ctypes.c_void_p

BRI17_OK = 0
STATUS = {
    0: "ok", 1: "invalid argument", 2: "unsupported size", 3: "CUDA error",
    4: "out of device memory", 5: "not converged", 6: "breakdown", 7: "no CUDA device",
    8: "busy", 9: "not found", 10: "cancelled",
    11: "a bounded device wait ran out (results invalid)", 12: "residual stagnated",
}
F64, F32 = 0, 1
CG_PLAIN, CG_MIXED, CG_MIXED_RESTART = 0, 1, 2


class CgInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("status", ctypes.c_int)]


class RequestResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int),
                ("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("submit_time_s", ctypes.c_double),
                ("admit_time_s", ctypes.c_double), ("finish_time_s", ctypes.c_double)]


class Bri17Error(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {STATUS.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


_SIGS = {
    "bri17_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "bri17_last_error": ([], ctypes.c_char_p),
    "bri17_version": ([], ctypes.c_char_p),
    "bri17_op_create": ([ctypes.c_int, c_int_p, c_double_p, ctypes.c_double, ctypes.c_double,
                         ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
    "bri17_op_destroy": ([vp], ctypes.c_int),
    "bri17_op_info": ([vp, c_int64_p, c_int64_p], ctypes.c_int),
    "bri17_op_set_material": ([vp, ctypes.c_double, ctypes.c_double], ctypes.c_int),
    "bri17_op_fused_form": ([vp, c_int_p], ctypes.c_int),
    "bri17_op_set_fused_form": ([vp, ctypes.c_int], ctypes.c_int),
    "bri17_wait_timeouts": ([c_int_p], ctypes.c_int),
    "bri17_op_sync_status": ([vp, vp], ctypes.c_int),
    "bri17_set_wait_limit_ns": ([ctypes.c_uint64], ctypes.c_int),
    "bri17_server_inject_alloc_failure": ([vp, ctypes.c_int], ctypes.c_int),
    "bri17_op_set_float_pair": ([vp, ctypes.c_int], ctypes.c_int),
    "bri17_eigenstress_to_opposite_strain": ([vp, vp, vp, vp], ctypes.c_int),
    "bri17_op_set_pass_timing": ([vp, ctypes.c_int], ctypes.c_int),
    "bri17_op_pass_times": ([vp, c_double_p, c_int64_p, ctypes.c_int, c_int_p], ctypes.c_int),
    "bri17_pass_name": ([ctypes.c_int], ctypes.c_char_p),
    "bri17_modal_stiffness_batch": ([vp, vp, ctypes.c_int64, vp, vp], ctypes.c_int),
    "bri17_modal_strain_displacement_batch": ([vp, vp, ctypes.c_int64, vp, vp], ctypes.c_int),
    "bri17_modal_eigenstress_to_opposite_strain_batch": (
        [vp, vp, ctypes.c_int64, vp, vp, vp], ctypes.c_int),
    "bri17_modal_stiffness_host": ([vp, vp, ctypes.c_int64, vp], ctypes.c_int),
    "bri17_modal_strain_displacement_host": ([vp, vp, ctypes.c_int64, vp], ctypes.c_int),
    "bri17_modal_eigenstress_to_opposite_strain_host": (
        [vp, vp, ctypes.c_int64, vp, vp], ctypes.c_int),
    "bri17_apply_stiffness": ([vp, vp, vp, vp], ctypes.c_int),
    "bri17_apply_stiffness_host": ([vp, vp, vp, vp], ctypes.c_int),
    "bri17_apply_stiffness_noalloc": ([ctypes.c_int, c_int_p, c_double_p, ctypes.c_double,
                                       ctypes.c_double, vp, vp, vp], ctypes.c_int),
    "bri17_apply_strain": ([vp, vp, vp, vp], ctypes.c_int),
    "bri17_eigenstress_rhs": ([vp, vp, vp, vp], ctypes.c_int),
    "bri17_cg_solve": ([vp, vp, vp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                        ctypes.POINTER(CgInfo), vp], ctypes.c_int),
    "bri17_server_create": ([ctypes.c_int64, ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
    "bri17_server_destroy": ([vp], ctypes.c_int),
    "bri17_server_set_size_priority": ([vp, ctypes.c_int], ctypes.c_int),
    "bri17_server_submit": ([vp, c_int_p, c_double_p, ctypes.c_double, ctypes.c_double,
                             vp, vp, ctypes.c_double, ctypes.c_int, c_int64_p], ctypes.c_int),
    "bri17_server_submit_borrowed": ([vp, c_int_p, c_double_p, ctypes.c_double, ctypes.c_double,
                             vp, vp, ctypes.c_double, ctypes.c_int, c_int64_p], ctypes.c_int),
    "bri17_server_step": ([vp, c_int_p], ctypes.c_int),
    "bri17_server_poll": ([vp, ctypes.POINTER(RequestResult), ctypes.c_int, c_int_p],
                          ctypes.c_int),
    "bri17_server_cancel": ([vp, ctypes.c_int64], ctypes.c_int),
    "bri17_server_clock": ([vp], ctypes.c_double),
}


def declared_symbols(header: str = HEADER):
    """Function names declared in the public header."""
    with open(header) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bri17_\w+)\s*\(", src)))


def load() -> ctypes.CDLL:
    """Load the library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: the CUDA library has not been built "
            "(run `python bri17_gb300/build.py`); there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(status: int, where: str) -> None:
    if status != BRI17_OK:
        detail = load().bri17_last_error().decode(errors="replace")
        raise Bri17Error(status, where, detail)
