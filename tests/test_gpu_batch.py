"""Batched mixed-precision pressure solves against the FP64 oracle.

The mixed solver stops on the FP64 true residual with the reference's own
rule, sqrt(eps/eps0) < qepsilon (1e-10).  Checked here:
  * that rule, re-evaluated on the CPU with the oracle's operators for the
    returned solution, is met (<= qepsilon);
  * qprecond 1 (the scaled system, whose mixed iterates track the FP64 ones):
    relative L2 <= 1e-9 against the oracle's solution at the same qepsilon,
    iteration count within 3% of the oracle's;
  * qprecond 0 and 2: the FP32 path drifts from the FP64 one, so the solution
    is compared with a tightly converged oracle solve (qepsilon 1e-13): its
    error is at most max(1e-9, 3x) the error of the oracle's own solve at
    qepsilon; iterations within +45%;
  * a problem's result does not depend on what else is in the batch
    (per-problem reductions in a fixed tile order): alone, mixed with others,
    split across several launches, or admitted while others run, the bits agree.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.batch import Batch, capacity_for
from suntans_gb300.capi import MAXITER, OK
from tests._cases import grid_cases, q_props, rel_l2, stopping_ratio

pytestmark = pytest.mark.gpu
TOL = 1e-9


def close_iters(n, m, qprecond=1):
    """qprecond 1 follows the FP64 iteration count; qprecond 0/2 need up to ~30%
    more iterations with FP32 vectors on stiff grids (measured; charged in the
    bench's 'equivalent' throughput)."""
    hi = 1.03 if qprecond == 1 else 1.45
    return m - max(3, int(0.03 * m)) <= n <= max(m + 3, int(hi * m) + 1)


@pytest.fixture(scope="module")
def oracle():
    return Oracle("port")


def tri_grids():
    return [
        gg.delaunay_seamount(600, 2000, 1000, Nkmax=15, sigma=300, ctop_frac=0.2, h_sigma=0.05, open_x0=False, seed=5),
        gg.delaunay_seamount(3000, 4000, 2000, Nkmax=30, sigma=500, rstretch=1.05, ctop_frac=0.05, h_sigma=0.02, seed=7),
        gg.delaunay_seamount(400, 1000, 500, Nkmax=6, H0=6.0, amp=5.5, sigma=150, ctop_frac=0.5, h_sigma=0.05, seed=11),
        gg.delaunay_seamount(1500, 3000, 1500, Nkmax=20, sigma=400, h_sigma=0.01, seed=13),
    ]


@pytest.mark.parametrize("form", [1, 2])
@pytest.mark.parametrize("qprecond", [0, 1, 2])
@pytest.mark.parametrize("gname", ["quad16x8", "quad64x16x32", "tri3000_partial", "tri400_shallow"])
def test_single_problem_matches_oracle(gpu_lib, oracle, qprecond, gname, form):
    g = dict(grid_cases())[gname]()
    prob = gg.make_q_problem(g, seed=1, q0_sigma=0.01)
    pr = q_props(qprecond)
    q_ref, n_ref = oracle.cgsolveq(prob, pr)
    b = Batch(qprecond=qprecond, maxfaces=g.maxfaces, **capacity_for([g]))
    b.set_fusion(form)
    i = b.add(prob, tol=pr.qepsilon, maxiters=pr.qmaxiters)
    running, ms, work = b.run()
    assert running == 0
    q, st = b.result(i, prob.q)
    assert st.status == OK
    assert close_iters(st.niters, n_ref, qprecond), (st.niters, n_ref)
    m = g.active_mask()
    check_accuracy(oracle, prob, q, q_ref, qprecond)
    assert np.array_equal(q[~m], prob.q[~m])
    b.close()


def check_accuracy(oracle, prob, q, q_ref, qprecond, tol=1e-10):
    m = prob.grid.active_mask()
    assert stopping_ratio(oracle, prob, q, qprecond) <= tol * (1 + 1e-6)
    if qprecond == 1:
        assert rel_l2(q, q_ref, m) <= TOL
    else:
        q_tight, _ = oracle.cgsolveq(prob, q_props(qprecond, qepsilon=1e-13, qmaxiters=40000))
        err_oracle = rel_l2(q_ref, q_tight, m)
        assert rel_l2(q, q_tight, m) <= max(TOL, 3 * err_oracle), (rel_l2(q, q_tight, m), err_oracle)


@pytest.mark.parametrize("qprecond", [0, 1, 2])
def test_batch_equals_solo_bitwise(gpu_lib, oracle, qprecond):
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=20 + k, q0_sigma=0.01) for k, g in enumerate(grids)]
    solo = []
    for g, p in zip(grids, probs):
        b = Batch(qprecond=qprecond, maxfaces=3, **capacity_for([g]))
        i = b.add(p, maxiters=4000)
        b.run()
        solo.append(b.result(i, p.q))
        b.close()
    b = Batch(qprecond=qprecond, maxfaces=3, **capacity_for(grids))
    ids = [b.add(p, maxiters=4000) for p in probs]
    running, ms, work = b.run()
    assert running == 0 and work > 0
    for k, (i, g, p) in enumerate(zip(ids, grids, probs)):
        q, st = b.result(i, p.q)
        assert st.niters == solo[k][1].niters
        assert np.array_equal(q, solo[k][0])
        q_ref, n_ref = oracle.cgsolveq(p, q_props(qprecond, qmaxiters=4000))
        check_accuracy(oracle, p, q, q_ref, qprecond)
        assert close_iters(st.niters, n_ref, qprecond)


def test_chunked_launches_and_late_admission(gpu_lib):
    """Continuous batching: launches of 5 iterations, a problem admitted while
    the others are mid-solve, finished problems released and their memory
    reused; every result equals its solo result bit for bit."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=40 + k) for k, g in enumerate(grids)]
    solo = []
    for g, p in zip(grids, probs):
        b = Batch(qprecond=1, maxfaces=3, **capacity_for([g]))
        i = b.add(p)
        b.run()
        solo.append(b.result(i, p.q))
        b.close()
    cap = capacity_for(grids[:3])
    b = Batch(qprecond=1, maxfaces=3, **cap)
    live = {b.add(probs[0]): 0, b.add(probs[1]): 1}
    pending = [2, 3]
    results = {}
    for step in range(10000):
        running, ms, work = b.run(max_iters=5)
        for i, k in list(live.items()):
            if b.state(i) == 3:
                results[k] = b.result(i, probs[k].q)
                del live[i]
        if pending and step >= 2:
            try:
                live[b.add(probs[pending[0]])] = pending[0]
                pending.pop(0)
            except Exception:
                pass  # arena full: admit once memory frees up
        if not live and not pending:
            break
    assert sorted(results) == [0, 1, 2, 3]
    for k in range(4):
        assert results[k][1].niters == solo[k][1].niters
        assert np.array_equal(results[k][0], solo[k][0])


def test_maxiter_status(gpu_lib):
    g = tri_grids()[0]
    p = gg.make_q_problem(g, seed=3)
    b = Batch(qprecond=0, maxfaces=3, **capacity_for([g]))
    i = b.add(p, maxiters=9)
    b.run()
    q, st = b.result(i, p.q)
    assert st.status == MAXITER and st.niters == 9
    assert np.all(np.isfinite(q))


def test_zero_rhs_done_without_iterations(gpu_lib):
    g = tri_grids()[2]
    p = gg.make_q_problem(g, seed=3)
    p.src[:] = 0.0
    b = Batch(qprecond=1, maxfaces=3, **capacity_for([g]))
    i = b.add(p)
    b.run()
    q, st = b.result(i, p.q)
    assert st.niters == 0 and st.status == OK and np.array_equal(q, p.q)


def test_resubmit_warm_start_matches_oracle(gpu_lib, oracle):
    """A finished problem re-submitted with a new right-hand side solves from
    its resident last solution (the model's phys->qc warm start)."""
    g = tri_grids()[0]
    p1 = gg.make_q_problem(g, seed=51)
    p2 = gg.make_q_problem(g, seed=52)
    b = Batch(qprecond=1, maxfaces=3, **capacity_for([g]))
    i = b.add(p1)
    b.run()
    q1, _ = b.result(i, p1.q, release=False)
    b.resubmit(i, p2.src)
    b.run()
    q2, st = b.result(i, p1.q)
    p2w = gg.QProblem(grid=g, D=p2.D, src=p2.src, q=q1, c=p2.c)
    q_ref, n_ref = oracle.cgsolveq(p2w, q_props(1))
    assert st.status == OK and close_iters(st.niters, n_ref, 1)
    check_accuracy(oracle, p2w, q2, q_ref, 1)


def test_graph_replay_equals_direct(gpu_lib):
    """Launches replayed from a CUDA graph give the same bits as direct ones."""
    grids = tri_grids()[:3]
    probs = [gg.make_q_problem(g, seed=60 + k) for k, g in enumerate(grids)]
    out = {}
    for mode in (False, True):
        b = Batch(qprecond=1, maxfaces=3, **capacity_for(grids))
        active = b.use_graph(mode)
        ids = [b.add(p) for p in probs]
        res = []
        for rep in range(3):
            b.run()
            res.append([b.result(i, p.q, release=False)[0] for i, p in zip(ids, probs)])
            for i, p in zip(ids, probs):
                b.resubmit(i, p.src, warm=False)
        out[mode] = (res, active, b.graph_launches())
        b.close()
    res_direct, _, _ = out[False]
    res_graph, active, launches = out[True]
    assert active and launches >= 2  # captured once, replayed for the unchanged set
    for ra, rb in zip(res_direct, res_graph):
        for a, c in zip(ra, rb):
            assert np.array_equal(a, c)


def test_overlapped_launch_wait_equals_solo(gpu_lib):
    """sgpu_batch_launch / sgpu_batch_wait: while a launch runs, finished
    problems are read back, new problems added and a finished problem
    re-submitted (a warm start on a new right-hand side); every result equals
    the same sequence run launch by launch, bit for bit."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=60 + k) for k, g in enumerate(grids)]
    p_re = gg.make_q_problem(grids[2], seed=70)

    def solo(k, resubmit=None):
        b = Batch(qprecond=1, maxfaces=3, **capacity_for([grids[k]]))
        i = b.add(probs[k])
        b.run()
        out = b.result(i, probs[k].q, release=False)
        if resubmit is not None:
            b.resubmit(i, resubmit.src)
            b.run()
            out = b.result(i, probs[k].q, release=False)
        b.close()
        return out

    ref = [solo(k) for k in range(4)]
    ref_re = solo(2, p_re)
    b = Batch(qprecond=1, maxfaces=3, **capacity_for(grids))
    live = {b.add(probs[2]): 2, b.add(probs[0]): 0}
    pending = [1, 3]
    results, resubmitted = {}, False
    b.launch(max_iters=5)
    for step in range(10000):
        # work while the launch runs
        done = [(i, k) for i, k in live.items() if b.state(i) == 3]
        for i, k in done:
            if k == 2 and not resubmitted:
                results["first2"] = b.result(i, probs[2].q, release=False)
                b.resubmit(i, p_re.src)
                resubmitted = True
                continue
            results[k] = b.result(i, probs[k].q, release=False)
            del live[i]
        if pending and step >= 1:
            k = pending.pop(0)
            live[b.add(probs[k])] = k
        running, ms, work = b.wait()
        if not live and not pending:
            break
        b.launch(max_iters=5)
    assert sorted(k for k in results if k != "first2") == [0, 1, 2, 3]
    for k in (0, 1, 3):
        assert results[k][1].niters == ref[k][1].niters and np.array_equal(results[k][0], ref[k][0])
    assert np.array_equal(results["first2"][0], ref[2][0])
    assert results[2][1].niters == ref_re[1].niters and np.array_equal(results[2][0], ref_re[0])
    b.close()


@pytest.mark.parametrize("qprecond", [0, 1, 2])
def test_fusion_forms_equal_bitwise(gpu_lib, qprecond):
    """The solution update run in the next apply pass (form 1, the default) or
    in the update pass (0): the same FP32 operations on the same operands, so
    the same bits and iteration counts; also across chunked launches (the
    increment deferred past a launch boundary and into the reliable updates),
    and MAXITER stops.  qprecond 2 runs the one-pass form (2) as form 1."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=60 + k, q0_sigma=0.01) for k, g in enumerate(grids)]
    out = {}
    for form in ((0, 1, 2) if qprecond == 2 else (0, 1)):
        for chunk in (0, 7):
            b = Batch(qprecond=qprecond, maxfaces=3, **capacity_for(grids))
            b.set_fusion(form)
            ids = [b.add(p, maxiters=4000 if k else 25) for k, p in enumerate(probs)]
            while True:
                running, _, _ = b.run(max_iters=chunk)
                if running == 0:
                    break
            out[(form, chunk)] = [b.result(i, p.q) for i, p in zip(ids, probs)]
            b.close()
    ref = out[(0, 0)]
    assert ref[0][1].status == MAXITER
    for key, res in out.items():
        for (q, st), (q0, st0) in zip(res, ref):
            assert st.status == st0.status and st.niters == st0.niters, key
            assert np.array_equal(q, q0), key


@pytest.mark.parametrize("qprecond", [0, 1])
def test_one_pass_form_matches_oracle(gpu_lib, oracle, qprecond):
    """The one-pass form (2): every problem meets the reference's stopping rule
    on the FP64 true residual and the accuracy bar of the two-pass form against
    the oracle, with iteration counts within the same bounds; its bits do not
    depend on chunked launches (the pending step and the buffer parity carried
    across launch boundaries and reliable updates) and a MAXITER stop is
    reported at the limit."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=80 + k, q0_sigma=0.01) for k, g in enumerate(grids)]
    pr = q_props(qprecond)
    out = {}
    for chunk in (0, 7):
        b = Batch(qprecond=qprecond, maxfaces=3, **capacity_for(grids))
        b.set_fusion(2)
        ids = [b.add(p, tol=pr.qepsilon, maxiters=25 if k == 0 else pr.qmaxiters) for k, p in enumerate(probs)]
        while True:
            running, _, _ = b.run(max_iters=chunk)
            if running == 0:
                break
        out[chunk] = [b.result(i, p.q) for i, p in zip(ids, probs)]
        b.close()
    for (q, st), (q0, st0) in zip(out[7], out[0]):
        assert st.status == st0.status and st.niters == st0.niters
        assert np.array_equal(q, q0)
    assert out[0][0][1].status == MAXITER and out[0][0][1].niters == 25
    for p, (q, st) in list(zip(probs, out[0]))[1:]:
        q_ref, n_ref = oracle.cgsolveq(p, pr)
        assert st.status == OK
        assert close_iters(st.niters, n_ref, qprecond), (st.niters, n_ref)
        check_accuracy(oracle, p, q, q_ref, qprecond)
        m = p.grid.active_mask()
        assert np.array_equal(q[~m], p.q[~m])


def test_one_pass_form_alone_equals_in_batch(gpu_lib):
    """A problem's one-pass solve does not depend on the rest of the batch."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=90 + k) for k, g in enumerate(grids)]
    b = Batch(qprecond=1, maxfaces=3, **capacity_for([grids[1]]))
    b.set_fusion(2)
    i = b.add(probs[1])
    b.run()
    alone = b.result(i, probs[1].q)
    b.close()
    b = Batch(qprecond=1, maxfaces=3, **capacity_for(grids))
    b.set_fusion(2)
    ids = [b.add(p) for p in probs]
    b.run()
    q, st = b.result(ids[1], probs[1].q)
    b.close()
    assert st.niters == alone[1].niters and np.array_equal(q, alone[0])


@pytest.mark.parametrize("form", [1, 2])
def test_stride_pauses_problems_without_changing_their_bits(gpu_lib, form):
    """A problem with stride s takes part in every s-th global iteration of a
    launch (the first launch of 12: strides 3 and 2 give 4 and 6 iterations,
    counted in the launch's work), and its result and iteration count are
    those of the unstrided batch, bit for bit; a stride may change in
    mid-solve."""
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=100 + k) for k, g in enumerate(grids)]
    N = [g.n_q() for g in grids]
    out = {}
    for strided in (False, True):
        b = Batch(qprecond=1, maxfaces=3, **capacity_for(grids))
        b.set_fusion(form)
        ids = [b.add(p) for p in probs]
        if strided:
            b.set_stride(ids[1], 3)
            b.set_stride(ids[2], 2)
        running, _, work = b.run(max_iters=12)
        assert running == len(probs)
        sweeps = [12, 4, 6, 12] if strided else [12] * 4
        if form == 1:
            assert work == sum(n * k for n, k in zip(N, sweeps)), (work, sweeps)
        else:
            # the one-pass form's first sweep forms the first direction and
            # counts no iteration (nor does a sweep after a reliable update)
            expect = sum(n * (k - 1) for n, k in zip(N, sweeps))
            assert expect - 2 * max(N) <= work <= expect, (work, expect)
        if strided:
            b.set_stride(ids[1], 1)  # changed in mid-solve
        while b.run()[0]:
            pass
        out[strided] = [b.result(i, p.q) for i, p in zip(ids, probs)]
        b.close()
    for (q, st), (q0, st0) in zip(out[True], out[False]):
        assert st.status == st0.status == OK and st.niters == st0.niters
        assert np.array_equal(q, q0)


def test_fusion_change_refused_mid_solve(gpu_lib):
    g = tri_grids()[1]
    b = Batch(qprecond=1, maxfaces=3, **capacity_for([g]))
    b.add(gg.make_q_problem(g, seed=3))
    b.run(max_iters=3)
    with pytest.raises(Exception):
        b.set_fusion(0)
    b.set_fusion(1)  # unchanged: accepted
    b.close()


def test_autotune_sweeps_the_three_knobs(gpu_lib):
    """CTAs per SM, slots per tile and the fusion of the solution update are
    all swept; the chosen shape is a measured, feasible one."""
    from suntans_gb300.autotune import autotune
    grids = tri_grids()
    probs = [gg.make_q_problem(g, seed=70 + k) for k, g in enumerate(grids)]
    best, table = autotune(probs, qprecond=1, iters=4, ctas_per_sm=(1, 2), tile_slots=(512, 1024))
    assert len(table) == 2 * 2 * 3
    assert {(r["ctas_per_sm"], r["tile_slots"], r["fusion"]) for r in table} == \
        {(c, t, f) for c in (1, 2) for t in (512, 1024) for f in (0, 1, 2)}
    assert best["rate"] > 0 and best["rate"] == max(r["rate"] for r in table)
