"""Continuous-batching server: every result equals its solo solve within
the stated tolerance (both are solved to 1e-8 relative residual, so they
agree to kappa * 1e-8 with the exact oracle solution), requests are admitted
while others run, cancellation and validation behave."""
import numpy as np
import pytest

from gpu_helpers import pair, rel_l2, to_dev
from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]

TOL = 1e-8
SOLUTION_TOL = 1e-5  # kappa (< 1e3 on these grids) * TOL, with margin


def _requests(rng, n, sides):
    reqs = []
    for i in range(n):
        s = sides[i % len(sides)]
        shape = (s, s, s) if isinstance(s, int) else s
        mu = float(rng.uniform(0.5, 2.0))
        nu = float(rng.uniform(0.1, 0.45))
        tau = rng.standard_normal((6,) + shape)
        reqs.append((shape, (1.0, 1.0, 1.0), mu, nu, tau))
    return reqs


def test_server_results_equal_solo_solves_and_oracle():
    from bri17_gb300.server import Server
    rng = np.random.default_rng(3)
    # (15, 15, 15) puts odd slot offsets in its bucket (unaligned vectors).
    reqs = _requests(rng, 10, [16, 24, (20, 16, 12), (15, 15, 15)])
    srv = Server(memory_budget_bytes=2 << 30, slots_per_bucket=4)
    ids = [srv.submit(*r, tol=TOL) for r in reqs]
    results = {r["id"]: r for r in srv.run_until_idle()}
    assert sorted(results) == sorted(ids)
    for rid, (shape, L, mu, nu, tau) in zip(ids, reqs):
        res = results[rid]
        assert res["status"] == 0, res
        assert res["rel_residual"] <= TOL
        x_srv = srv.result(rid)
        h, ho = pair(shape, L, mu, nu)
        b = h.eigenstress_rhs(to_dev(tau))
        x_solo, info = h.cg_solve(b, tol=TOL, mode="mixed")
        # Same algorithm alone and in the mix: similar work.
        assert res["iterations"] <= 1.5 * info["iterations"] + 32, (res, info)
        x_ref = O.eigenstress_solve(ho, tau)
        assert rel_l2(x_srv, x_solo.cpu().numpy()) <= SOLUTION_TOL
        assert rel_l2(x_srv, x_ref) <= SOLUTION_TOL
        # True FP64 residual of the served solution.
        r = b - h.apply_stiffness(to_dev(x_srv))
        assert float(r.norm() / b.norm()) <= 1.01 * TOL
    srv.close()


def test_served_results_equal_solo_solves_at_benchmark_sides():
    """The same check at sides of the serving benchmark (32 and 48, cubic,
    L = 1), several requests per bucket mixed with another geometry: each
    served solution equals its solo mixed solve and the FP64 oracle within
    the stated tolerance."""
    from bri17_gb300.server import Server
    rng = np.random.default_rng(13)
    reqs = _requests(rng, 6, [32, 48])
    srv = Server(memory_budget_bytes=4 << 30, slots_per_bucket=8)
    ids = [srv.submit(*r, tol=TOL) for r in reqs]
    results = {r["id"]: r for r in srv.run_until_idle()}
    for rid, (shape, L, mu, nu, tau) in zip(ids, reqs):
        res = results[rid]
        assert res["status"] == 0 and res["rel_residual"] <= TOL, res
        x_srv = srv.result(rid)
        h, ho = pair(shape, L, mu, nu)
        b = h.eigenstress_rhs(to_dev(tau))
        x_solo, info = h.cg_solve(b, tol=TOL, mode="mixed")
        x_ref = O.eigenstress_solve_half(ho, tau, workers=4)
        assert rel_l2(x_srv, x_solo.cpu().numpy()) <= SOLUTION_TOL
        assert rel_l2(x_srv, x_ref) <= SOLUTION_TOL
    srv.close()


def test_requests_are_admitted_while_others_run():
    """Two slots, five requests of one size: later requests enter slots freed
    by earlier ones while the other slot is still solving."""
    from bri17_gb300.server import Server
    rng = np.random.default_rng(4)
    reqs = _requests(rng, 5, [16])
    srv = Server(memory_budget_bytes=1 << 30, slots_per_bucket=2)
    ids = [srv.submit(*r, tol=TOL) for r in reqs]
    results = {r["id"]: r for r in srv.run_until_idle()}
    assert all(results[i]["status"] == 0 for i in ids)
    admits = sorted(results[i]["admit_time_s"] for i in ids)
    finishes = sorted(results[i]["finish_time_s"] for i in ids)
    # The third admission happens once the first solve has left its slot
    # (its finish time is stamped when the asynchronous copy of its solution
    # has landed, a little later) and before the last finish.
    assert admits[2] >= finishes[0] - 2e-3 and admits[2] < finishes[-1]
    overlap = any(results[a]["admit_time_s"] < results[b]["finish_time_s"] and
                  results[b]["admit_time_s"] < results[a]["finish_time_s"]
                  for a in ids for b in ids if a != b)
    assert overlap
    srv.close()


def test_cancel_queued_and_running():
    from bri17_gb300.server import Server
    rng = np.random.default_rng(5)
    reqs = _requests(rng, 3, [24])
    srv = Server(memory_budget_bytes=1 << 30, slots_per_bucket=1)
    ids = [srv.submit(*r, tol=1e-12, max_iterations=100000) for r in reqs]
    srv.step()                      # first request admitted and running
    assert srv.cancel(ids[2]) == 0  # still queued
    assert srv.cancel(ids[0]) == 0  # running
    assert srv.cancel(999999) == 9  # unknown id
    results = {r["id"]: r for r in srv.run_until_idle()}
    assert results[ids[2]]["status"] == 10
    assert results[ids[0]]["status"] == 10
    assert results[ids[1]]["status"] == 0
    srv.close()


def test_submit_validation():
    from bri17_gb300._lib import Bri17Error
    from bri17_gb300.server import Server
    srv = Server(memory_budget_bytes=64 << 20, slots_per_bucket=2)
    tau = np.zeros((6, 8, 8, 8))
    with pytest.raises(Bri17Error):
        srv.submit((8, 8, 8), (1, 1, 1), 1.0, 0.5, tau)      # nu = 0.5
    with pytest.raises(Bri17Error):
        srv.submit((256, 256, 256), (1, 1, 1), 1.0, 0.3, np.zeros(6 * 256 ** 3))
    with pytest.raises(Bri17Error):
        srv.submit((8, 8, 8), (1, float("inf"), 1), 1.0, 0.3, tau)  # non-finite L
    with pytest.raises(Bri17Error):
        srv.submit((8, 8, 8), (1, 1, 1), float("inf"), 0.3, tau)  # non-finite mu
    import ctypes

    from bri17_gb300 import _lib
    n = ctypes.c_int()
    assert _lib.load().bri17_server_poll(srv._h, (_lib.RequestResult * 1)(), -1,
                                         ctypes.byref(n)) == 1   # negative cap
    rid = srv.submit((8, 8, 8), (1, 1, 1), 1.0, 0.3, tau)  # tau = 0 -> x = 0
    res = srv.run_until_idle()
    assert res[0]["status"] == 0 and np.all(srv.result(rid) == 0)
    srv.close()


def test_idle_bucket_released_when_memory_is_needed():
    """With a budget that holds one bucket, a second geometry is admitted
    after the first one's requests finish (its bucket is released)."""
    from bri17_gb300.server import Server
    rng = np.random.default_rng(6)
    # A 48^3 bucket of 2 slots needs about 52 MB, a 40^3 one about 30 MB:
    # a 70 MB budget holds either, not both.
    a = _requests(rng, 2, [48])
    b = _requests(rng, 2, [40])
    srv = Server(memory_budget_bytes=70 << 20, slots_per_bucket=2)
    ids = [srv.submit(*r, tol=TOL) for r in a + b]
    results = {r["id"]: r for r in srv.run_until_idle()}
    assert all(results[i]["status"] == 0 for i in ids)
    # The second geometry was admitted only after the first one's solves had
    # left their slots (finish times are stamped when the asynchronous
    # copies of the solutions have landed, a little later).
    assert min(results[i]["admit_time_s"] for i in ids[2:]) >= \
        max(results[i]["finish_time_s"] for i in ids[:2]) - 2e-3
    srv.close()


def test_copying_submit_with_pageable_buffers():
    """bri17_server_submit (tau copied at submit, pageable x) gives the same
    solutions as the borrowed page-locked path of Server.submit."""
    import ctypes

    from bri17_gb300 import _lib
    from bri17_gb300.server import Server
    rng = np.random.default_rng(7)
    reqs = _requests(rng, 3, [16, 12])
    srv = Server(memory_budget_bytes=1 << 30, slots_per_bucket=2)
    borrowed = [srv.submit(*r, tol=TOL) for r in reqs]
    xs, copied = [], []
    for shape, L, mu, nu, tau in reqs:
        x = np.zeros((3,) + shape)
        rid = ctypes.c_int64()
        t = np.ascontiguousarray(tau)
        assert _lib.load().bri17_server_submit(
            srv._h, (ctypes.c_int * 3)(*shape), (ctypes.c_double * 3)(*L), mu, nu,
            t.ctypes.data_as(ctypes.c_void_p), x.ctypes.data_as(ctypes.c_void_p), TOL, 100000,
            ctypes.byref(rid)) == 0
        del t  # copied at submit
        xs.append(x)
        copied.append(rid.value)
        srv.pending += 1
    results = {r["id"]: r for r in srv.run_until_idle()}
    for b, c, x in zip(borrowed, copied, xs):
        assert results[b]["status"] == 0 and results[c]["status"] == 0
        assert np.array_equal(srv.result(b), x)
    srv.close()


def test_served_results_at_a_float_pair_side():
    """Side 128 (the serving benchmark's largest): its bucket computes each
    slot's FP64 residual in float pairs with that slot's material (the
    float-pair axis-0 pass with in-tile exchanges), beside a 32^3 bucket
    on the FP64 pipe.  Each served solution equals its solo mixed solve and
    the FP64 oracle within the stated tolerance, and its true FP64 residual
    meets the tolerance."""
    from bri17_gb300.server import Server
    rng = np.random.default_rng(29)
    reqs = _requests(rng, 3, [128, 32, 128])
    srv = Server(memory_budget_bytes=4 << 30, slots_per_bucket=2)
    ids = [srv.submit(*r, tol=TOL) for r in reqs]
    results = {r["id"]: r for r in srv.run_until_idle()}
    assert sorted(results) == sorted(ids)
    for rid, (shape, L, mu, nu, tau) in zip(ids, reqs):
        res = results[rid]
        assert res["status"] == 0 and res["rel_residual"] <= TOL, res
        x_srv = srv.result(rid)
        h, ho = pair(shape, L, mu, nu)
        b = h.eigenstress_rhs(to_dev(tau))
        x_solo, info = h.cg_solve(b, tol=TOL, mode="mixed")
        x_ref = O.eigenstress_solve_half(ho, tau, workers=4)
        assert rel_l2(x_srv, x_solo.cpu().numpy()) <= SOLUTION_TOL
        assert rel_l2(x_srv, x_ref) <= SOLUTION_TOL
        r = b - h.apply_stiffness(to_dev(x_srv))
        assert float(r.norm() / b.norm()) <= 1.01 * TOL
    srv.close()
