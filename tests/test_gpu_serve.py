"""Serving loop on the GPU: continuous batching over the batched solver.

* Every result is the same alone and in the mix: the same requests served one
  at a time (each alone on the device) and all admitted together (overlapping
  in shared launches, admitted between launches as others finish) give the
  same bits.  The stated tolerance is exact equality: the batched kernel's
  reductions run in a fixed per-problem order.
* Warm starts: a repeated request on a resident grid starts from the grid's
  previous solution and meets the reference's stopping rule (re-evaluated on
  the CPU with the oracle's operators) for its own tolerance.
* A tight HBM budget forces evictions and cold restarts; every result still
  meets its stopping rule from the initial guess it used.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.batch import Batch, capacity_for, request_bytes
from suntans_gb300.serve import Request, Server, request_src
from tests._cases import stopping_ratio

pytestmark = pytest.mark.gpu

SEQ = [0, 1, 2, 1, 0, 2, 2, 1, 0, 0, 1, 2]


def small_pool():
    return gg.serving_pool(n=3, seed=21, nc_range=(1500, 5000), nkmax_range=(8, 20), rhs_per_grid=2)


def stream():
    """Requests whose right-hand sides all differ: with the reference's relative
    stopping rule, a warm start from the solution of the very same right-hand
    side would have to push the residual below round-off."""
    tols = (1e-8, 1e-10)
    reqs = [Request(k, g, (k // 3) % 2, tols[k % 2], 0.001 * k, mix=0.03 * k) for k, g in enumerate(SEQ)]
    w = [1 - r.mix if r.rhs == 0 else r.mix for r in reqs]  # weight of the first stored right-hand side
    assert min(abs(a - b) for i, a in enumerate(w) for b in w[:i]) > 0.02
    return reqs


def serve(pool, reqs, one_at_a_time, budget=1e12, chunk=16, copies=1):
    grids = [p[0].grid for p in pool]
    b = Batch(qprecond=1, maxfaces=3, **capacity_for(grids * copies))
    b.use_graph(True)
    srv = Server(pool, b, budget, lambda g: request_bytes(g, 1), chunk=chunk, keep_q=True, copies=copies)
    if one_at_a_time:
        for r in reqs:
            srv.run([r], realtime=False)
    else:
        srv.run(reqs, realtime=False)
    b.close()
    return reqs, srv


def check_chain(pool, reqs):
    """Each result meets the reference's stopping rule for its tolerance from the
    initial guess it used: the solution of request `warm_from` when warm (the
    previous request on the same resident copy of its grid, or the grid's
    latest one for a new copy), else cold."""
    o = Oracle("port")
    by_rid = {r.rid: r for r in reqs}
    for r in reqs:
        assert r.status == 0
        p = pool[r.grid][r.rhs]
        q0 = by_rid[r.warm_from].q if r.warm else p.q
        pw = gg.QProblem(grid=p.grid, D=p.D, src=request_src(pool, r), q=q0, c=p.c)
        assert stopping_ratio(o, pw, r.q, 1) <= r.tol * 1.0001


def test_same_alone_and_in_mix(gpu_lib):
    pool = small_pool()
    alone, _ = serve(pool, stream(), True)
    mixed, srv = serve(pool, stream(), False, chunk=7)
    assert srv.launches > 1
    assert max(r.launch_done for r in mixed) > min(r.launch_done for r in mixed)
    for a, m in zip(alone, mixed):
        assert a.status == 0 and m.status == 0
        assert a.iters == m.iters
        assert np.array_equal(a.q, m.q)


def test_warm_start_chain_meets_stopping_rule(gpu_lib):
    pool = small_pool()
    reqs, srv = serve(pool, stream(), False)
    assert srv.evictions == 0
    assert [r.warm for r in reqs] == [k >= 3 for k in range(len(SEQ))]  # first visit of each grid is cold
    check_chain(pool, reqs)


def test_tight_budget_evicts_and_stays_correct(gpu_lib):
    pool = small_pool()
    sizes = sorted(request_bytes(p[0].grid, 1) for p in pool)
    reqs, srv = serve(pool, stream(), False, budget=sizes[-1] + sizes[-2])  # two grids resident at most
    assert srv.evictions > 0
    assert not all(r.warm for r in reqs[3:])  # some revisits found their grid evicted
    check_chain(pool, reqs)


def test_copies_of_hot_grids_meet_stopping_rule(gpu_lib):
    """Two resident copies per grid: requests on a busy grid run at once on a
    second copy; each result still solves its own request to its tolerance
    from the initial guess it was given (the same within the tolerance as
    served alone, not the same bits)."""
    pool = small_pool()
    reqs, srv = serve(pool, stream(), False, copies=2)
    assert max(r.copy for r in reqs) == 1
    assert max(srv.ncopy.values()) == 2
    check_chain(pool, reqs)
