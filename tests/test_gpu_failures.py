"""Failure detection without a GPU fault.

* A bounded device wait that runs out reaches the caller as
  BRI17_ERR_TIMEOUT (11): the wait limit of the tensor-copy kernels is set
  to 0 (diagnostics), so their first wait on a tile's copies gives up at
  once; the kernel still waits, with the normal one-second limit, for its
  own copies to land before it leaves, then reports through the handle's
  status words.  The handle works again once the limit is back at its
  default.
* A bucket the server cannot allocate fails only the request that needed
  it (BRI17_ERR_OUT_OF_MEMORY, 4), injected on the host; the requests in
  flight finish bit-identically to a run without the failure.
* A tolerance below what the FP64 residual resolves ends the solve with
  BRI17_ERR_STAGNATED (12) instead of running to the iteration cap.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from gpu_helpers import pair, rel_l2, to_dev
from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]

TIMEOUT, OOM, STAGNATED = 11, 4, 12
DEFAULT_LIMIT_NS = 1_000_000_000
SHAPE32 = (64, 32, 32)  # even shape[1]: the FP32 TMA-staged axis-0 form applies


@pytest.fixture
def zero_wait_limit():
    """Call the yielded function (after creating the handles, whose FP32
    form timing must run at the normal limit) to set the limit to 0; the
    default is restored at the end."""
    from bri17_gb300 import set_wait_limit_ns, wait_timeouts

    def zero():
        import torch
        torch.cuda.synchronize()
        wait_timeouts()  # clear the device counters
        set_wait_limit_ns(0)
    try:
        yield zero
    finally:
        import torch
        torch.cuda.synchronize()
        set_wait_limit_ns(DEFAULT_LIMIT_NS)
        wait_timeouts()  # the counts this test made are not left for later tests


def _tma_handle():
    h, ho = pair(SHAPE32, (1.0, 1.0, 1.0), 1.0, 0.3, precision="f32")
    h.fused_form = "tma"
    return h, ho


def test_run_out_wait_is_reported_by_sync_status_and_next_call(zero_wait_limit):
    import ctypes

    import torch

    from bri17_gb300 import _lib, set_wait_limit_ns, wait_timeouts
    h, ho = _tma_handle()
    u = np.random.default_rng(1).standard_normal((3,) + SHAPE32)
    ud = to_dev(u, torch.float32)
    f = torch.empty_like(ud)
    L = _lib.load()
    assert h.sync_status() == 0
    zero_wait_limit()
    # Stream-ordered call: returns before its kernels run.
    assert L.bri17_apply_stiffness(h.handle, ctypes.c_void_p(ud.data_ptr()),
                                   ctypes.c_void_p(f.data_ptr()), None) == 0
    assert h.sync_status() == TIMEOUT
    assert b"ran out" in L.bri17_last_error()
    assert h.sync_status() == 0  # reported once
    assert wait_timeouts() > 0
    # Reported by the next field call, which then enqueues nothing.
    assert L.bri17_apply_stiffness(h.handle, ctypes.c_void_p(ud.data_ptr()),
                                   ctypes.c_void_p(f.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert L.bri17_apply_stiffness(h.handle, ctypes.c_void_p(ud.data_ptr()),
                                   ctypes.c_void_p(f.data_ptr()), None) == TIMEOUT
    # Back at the default limit the handle computes correctly again.
    set_wait_limit_ns(DEFAULT_LIMIT_NS)
    wait_timeouts()
    f = h.apply_stiffness(ud)
    assert h.sync_status() == 0 and wait_timeouts() == 0
    f_ref = O.apply_stiffness(ho, u.astype(np.float32).astype(np.float64))
    assert rel_l2(f.cpu().numpy(), f_ref) <= 2e-5


def test_run_out_wait_fails_the_synchronous_entry_points(zero_wait_limit):
    import torch

    from bri17_gb300 import set_wait_limit_ns
    from bri17_gb300._lib import Bri17Error
    h, ho = _tma_handle()
    u = np.random.default_rng(2).standard_normal((3,) + SHAPE32).astype(np.float32)
    tau = np.random.default_rng(3).standard_normal((6,) + SHAPE32)
    h64, _ = pair(SHAPE32, (1.0, 1.0, 1.0), 1.0, 0.3)
    b = h64.eigenstress_rhs(to_dev(tau))
    assert h.sync_status() == 0
    zero_wait_limit()
    with pytest.raises(Bri17Error) as e:
        h.apply_stiffness_host(u)
    assert e.value.status == TIMEOUT
    # Plain CG on the FP32 handle: the first chunk's wait runs out.
    x, info = h.cg_solve(b, tol=1e-5, raise_on_failure=False)
    assert info["status"] == TIMEOUT, info
    set_wait_limit_ns(DEFAULT_LIMIT_NS)
    x, info = h.cg_solve(b, tol=1e-5)
    assert info["status"] == 0
    torch.cuda.synchronize()


def test_run_out_wait_in_the_float_pair_pass(zero_wait_limit):
    """The float-pair TMA axis-0 pass (in-tile exchanges at n0 = 64) reports
    a wait that ran out as the FP32 pass does: the handle's status is
    BRI17_ERR_TIMEOUT once, the device count is non-zero, and back at the
    default limit the float-pair result is within the FP64 bound of the
    oracle again."""
    import ctypes

    import torch

    from bri17_gb300 import _lib, set_wait_limit_ns, wait_timeouts
    shape = (64, 64, 128)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.25)
    h.set_float_pair(True)
    h.fused_form = "tma"
    u = np.random.default_rng(5).standard_normal((3,) + shape)
    u -= u.mean(axis=(1, 2, 3), keepdims=True)
    ud = to_dev(u)
    f = torch.empty_like(ud)
    L = _lib.load()
    assert h.sync_status() == 0
    zero_wait_limit()
    assert L.bri17_apply_stiffness(h.handle, ctypes.c_void_p(ud.data_ptr()),
                                   ctypes.c_void_p(f.data_ptr()), None) == 0
    assert h.sync_status() == TIMEOUT
    assert h.sync_status() == 0  # reported once
    assert wait_timeouts() > 0
    set_wait_limit_ns(DEFAULT_LIMIT_NS)
    wait_timeouts()
    f = h.apply_stiffness(ud)
    assert h.sync_status() == 0 and wait_timeouts() == 0
    assert rel_l2(f.cpu().numpy(), O.apply_stiffness(ho, u)) <= 1e-12


_SERVER_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from bri17_gb300 import set_wait_limit_ns
from bri17_gb300.server import Server
srv = Server(memory_budget_bytes=2 << 30, slots_per_bucket=4)
tau = np.random.default_rng(4).standard_normal((6, 32, 32, 32))
# Warm the bucket at the default limit, then make the chunks' waits run out.
srv.submit((32, 32, 32), (1, 1, 1), 1.0, 0.3, tau, tol=1e-8)
first = srv.run_until_idle()
set_wait_limit_ns(0)
srv.submit((32, 32, 32), (1, 1, 1), 1.0, 0.3, tau, tol=1e-8)
second = srv.run_until_idle()
set_wait_limit_ns(1_000_000_000)
srv.submit((32, 32, 32), (1, 1, 1), 1.0, 0.3, tau, tol=1e-8)
third = srv.run_until_idle()
print(first[0]["status"], second[0]["status"], third[0]["status"])
"""


def test_run_out_wait_fails_the_served_requests_of_that_chunk():
    """The server's buckets pick their axis-0 form by timing; the child
    process forces the tensor-copy form, so that every chunk's waits can run
    out."""
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, BRI17_FUSED_FORM="tma")
    p = subprocess.run([sys.executable, "-c", _SERVER_CHILD, repo], env=env,
                       capture_output=True, text=True, timeout=240)
    assert p.returncode == 0, p.stderr
    assert p.stdout.split() == ["0", str(TIMEOUT), "0"], p.stdout


def test_failed_bucket_allocation_fails_only_its_request():
    from bri17_gb300.server import Server
    rng = np.random.default_rng(5)
    tau_a = rng.standard_normal((6, 16, 16, 16))
    tau_b = rng.standard_normal((6, 20, 20, 20))

    def run(inject):
        srv = Server(memory_budget_bytes=2 << 30, slots_per_bucket=4)
        a = srv.submit((16, 16, 16), (1, 1, 1), 1.2, 0.3, tau_a, tol=1e-8)
        srv.step()  # a's bucket exists and a is in flight
        if inject:
            srv.inject_alloc_failure(3)  # after three buffers of the new bucket
        b = srv.submit((20, 20, 20), (1, 1, 1), 0.9, 0.25, tau_b, tol=1e-8)
        res = {r["id"]: r for r in srv.run_until_idle()}
        xa = np.array(srv.result(a))
        out = (res[a], xa, res[b])
        # The server keeps working: the same geometry gets its bucket now.
        srv.submit((20, 20, 20), (1, 1, 1), 0.9, 0.25, tau_b, tol=1e-8)
        res_c = srv.run_until_idle()
        srv.close()
        return out + (res_c[0],)

    ra, xa, rb, rc = run(inject=True)
    ra0, xa0, rb0, _ = run(inject=False)
    assert rb["status"] == OOM and rb0["status"] == 0
    assert ra["status"] == 0 and rc["status"] == 0
    assert np.array_equal(xa, xa0)  # bit-identical to the run without the failure
    assert ra["iterations"] == ra0["iterations"]


@pytest.mark.parametrize("mode", ["mixed", "plain"])
def test_unreachable_tolerance_reports_stagnation(mode):
    shape = (16, 16, 16)
    h, ho = pair(shape, (1.0, 1.0, 1.0), 1.0, 0.3)
    tau = np.random.default_rng(6).standard_normal((6,) + shape)
    b = h.eigenstress_rhs(to_dev(tau))
    x, info = h.cg_solve(b, tol=1e-17, max_iterations=20000, mode=mode,
                         raise_on_failure=False)
    assert info["status"] == STAGNATED, info
    assert info["iterations"] < 20000
    # The iterate is as good as FP64 allows.
    assert rel_l2(x.cpu().numpy(), O.eigenstress_solve(ho, tau)) <= 1e-11
