"""Python binding of the continuous-batching solve server
(``bri17_server_*`` in include/bri17_gb300.h).

    srv = Server(memory_budget_bytes=8 << 30, slots_per_bucket=8)
    rid = srv.submit(shape, L, mu, nu, tau)      # tau: (6, *shape) float64
    while srv.pending:
        srv.step()
        for res in srv.poll():
            x = srv.result(res["id"])             # (3, *shape) float64
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check


def _pinned_torch():
    """torch when page-locked host memory is available, else None."""
    try:
        import torch
    except ImportError:
        return None
    return torch if torch.cuda.is_available() else None


class Server:
    def __init__(self, memory_budget_bytes: int = 8 << 30, slots_per_bucket: int = 64,
                 size_priority: bool = False):
        """size_priority: smaller geometries on higher-priority streams (lower
        latency for small requests, lower throughput)."""
        L = _lib.load()
        h = ctypes.c_void_p()
        check(L.bri17_server_create(int(memory_budget_bytes), int(slots_per_bucket),
                                    ctypes.byref(h)), "bri17_server_create")
        self._h = h
        if size_priority:
            check(L.bri17_server_set_size_priority(h, 1), "bri17_server_set_size_priority")
        self._out = {}     # id -> solution array (kept alive until read)
        self._taus = {}
        self.pending = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().bri17_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clock(self) -> float:
        return _lib.load().bri17_server_clock(self._h)

    def submit(self, shape, L, mu, nu, tau, tol=1e-8, max_iterations=100000) -> int:
        """Queue one solve.  tau (numpy array or CPU tensor, (6, *shape)) is
        copied into page-locked memory held until the request is polled -- a
        page-locked float64 tensor is borrowed without a copy -- and the
        solution lands in a page-locked array, so the server's uploads and
        downloads are asynchronous (bri17_server_submit_borrowed)."""
        shape = tuple(int(n) for n in shape)
        if len(shape) != 3:
            raise ValueError("the server solves 3D problems")
        torch = _pinned_torch()
        if torch is not None and isinstance(tau, torch.Tensor):
            # A page-locked float64 CPU tensor is borrowed as it is.
            if tau.is_cuda:
                raise ValueError("tau must be host memory")
            tau = tau if (tau.dtype == torch.float64 and tau.is_contiguous()
                          and tau.is_pinned()) else tau.to(torch.float64).contiguous().numpy()
        else:
            tau = np.ascontiguousarray(tau, dtype=np.float64)
        count = tau.size if isinstance(tau, np.ndarray) else tau.numel()
        if count != 6 * int(np.prod(shape)):
            raise ValueError("tau must hold 6 x prod(shape) values")
        rid = ctypes.c_int64()
        args = ((ctypes.c_int * 3)(*shape), (ctypes.c_double * 3)(*L), float(mu), float(nu))
        if torch is not None:
            tau_t = tau if isinstance(tau, torch.Tensor) else torch.from_numpy(tau).pin_memory()
            x_t = torch.zeros((3,) + shape, dtype=torch.float64, pin_memory=True)
            check(_lib.load().bri17_server_submit_borrowed(
                self._h, *args, ctypes.c_void_p(tau_t.data_ptr()),
                ctypes.c_void_p(x_t.data_ptr()), float(tol), int(max_iterations),
                ctypes.byref(rid)), "bri17_server_submit_borrowed")
            self._taus[rid.value] = tau_t
            self._out[rid.value] = (x_t, x_t.numpy())
        else:
            x = np.zeros((3,) + shape)
            check(_lib.load().bri17_server_submit(
                self._h, *args, tau.ctypes.data_as(ctypes.c_void_p),
                x.ctypes.data_as(ctypes.c_void_p), float(tol), int(max_iterations),
                ctypes.byref(rid)), "bri17_server_submit")
            self._out[rid.value] = (None, x)
        self.pending += 1
        return rid.value

    def step(self) -> int:
        active = ctypes.c_int()
        check(_lib.load().bri17_server_step(self._h, ctypes.byref(active)), "bri17_server_step")
        return active.value

    def poll(self, cap: int = 256):
        buf = (_lib.RequestResult * cap)()
        n = ctypes.c_int()
        check(_lib.load().bri17_server_poll(self._h, buf, cap, ctypes.byref(n)),
              "bri17_server_poll")
        out = []
        for i in range(n.value):
            r = buf[i]
            out.append({"id": r.id, "status": r.status, "iterations": r.iterations,
                        "outer_iterations": r.outer_iterations,
                        "rel_residual": r.rel_residual, "submit_time_s": r.submit_time_s,
                        "admit_time_s": r.admit_time_s, "finish_time_s": r.finish_time_s})
        self.pending -= len(out)
        for r in out:
            self._taus.pop(r["id"], None)  # borrowed until the request is returned
        return out

    def result(self, rid: int) -> np.ndarray:
        return self._out.pop(rid)[1]

    def inject_alloc_failure(self, at: int) -> None:
        """Fault injection: the next bucket creation fails at its work
        buffer number `at` as if device memory had run out (-1 cancels);
        the request that needed the bucket finishes with status 4 (out of
        memory) and the others are unaffected."""
        check(_lib.load().bri17_server_inject_alloc_failure(self._h, int(at)),
              "bri17_server_inject_alloc_failure")

    def cancel(self, rid: int) -> int:
        return _lib.load().bri17_server_cancel(self._h, int(rid))

    def run_until_idle(self, max_steps: int = 1_000_000):
        results = []
        for _ in range(max_steps):
            if self.pending == 0:
                break
            self.step()
            results.extend(self.poll())
        return results
