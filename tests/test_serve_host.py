"""Scheduling logic of the serving loop (suntans_gb300/serve.py) on a host fake
of the batched engine: arrival order, one request per grid at a time, HBM
budget admission with least-recently-used eviction, warm starts on resident
grids, continuous admission between launches."""
import types

import numpy as np
import pytest

from suntans_gb300.capi import OOM, SolverError
from suntans_gb300.serve import PrefetchedSources, Request, Server, latency_report, poisson_stream, request_src


class FakeEngine:
    """Same methods as Batch; a problem needs 40 iterations cold (80 at 1e-10),
    a quarter of that warm.  Capacity counted in storage slots."""

    def __init__(self, cap):
        self.cap, self.used, self.inst, self.next = cap, 0, {}, 0
        self.peak = 0

    @staticmethod
    def _iters(tol, warm):
        n = 80 if tol < 1e-9 else 40
        return n // 4 if warm else n

    def add(self, prob, tol, maxiters):
        n = prob.grid.n3
        if self.used + n > self.cap:
            raise SolverError(OOM, "full")
        i = self.next
        self.next += 1
        self.inst[i] = dict(n=n, left=self._iters(tol, False), state=1, it=0)
        self.used += n
        self.peak = max(self.peak, self.used)
        return i

    def resubmit(self, i, src, tol, maxiters, warm):
        I = self.inst[i]
        assert I["state"] == 3
        I.update(left=self._iters(tol, warm), state=1, it=0)

    def run(self, max_iters=0):
        work, running = 0, 0
        for I in self.inst.values():
            if I["state"] in (1, 2):
                k = I["left"] if max_iters <= 0 else min(I["left"], max_iters)
                I["left"] -= k
                I["it"] += k
                work += k * I["n"]
                I["state"] = 3 if I["left"] == 0 else 2
                running += I["state"] != 3
        return running, 0.1, work

    def state(self, i):
        return self.inst[i]["state"]

    def result(self, i, q0, release=False, out=None):
        I = self.inst[i]
        st = types.SimpleNamespace(niters=I["it"], status=0, unknowns=I["n"])
        if release:
            self.release(i)
        return None, st

    def release(self, i):
        self.used -= self.inst.pop(i)["n"]


class FakeAsyncEngine(FakeEngine):
    """FakeEngine with the batched engine's launch / wait split: a launch runs
    the problems active when it is enqueued; their state changes only at wait,
    and adds, re-submissions and read-backs meanwhile touch other problems."""

    def __init__(self, cap):
        super().__init__(cap)
        self.pending = None

    def launch(self, max_iters=0):
        assert self.pending is None, "one launch in flight at a time"
        self.pending = ([i for i, I in self.inst.items() if I["state"] in (1, 2)], max_iters)

    def wait(self):
        if self.pending is None:
            return 0, 0.0, 0
        ids, max_iters = self.pending
        self.pending = None
        work, running = 0, 0
        for i in ids:
            I = self.inst[i]
            k = I["left"] if max_iters <= 0 else min(I["left"], max_iters)
            I["left"] -= k
            I["it"] += k
            work += k * I["n"]
            I["state"] = 3 if I["left"] == 0 else 2
            running += I["state"] != 3
        return running, (0.1 if ids else 0.0), work

    def resubmit(self, i, src, tol, maxiters, warm):
        assert self.pending is None or i not in self.pending[0]
        super().resubmit(i, src, tol, maxiters, warm)

    def result(self, i, q0, release=False, out=None):
        assert self.pending is None or i not in self.pending[0]
        return super().result(i, q0, release, out)

    def release(self, i):
        assert self.pending is None or i not in self.pending[0]
        super().release(i)


ENGINES = [FakeEngine, FakeAsyncEngine]


def fake_pool(sizes, rhs=2):
    pool = []
    for gid, n in enumerate(sizes):
        g = types.SimpleNamespace(n3=n, gid=gid)  # n3: storage slots
        pool.append([types.SimpleNamespace(grid=g, src=np.full(3, float(j + 1)), q=None) for j in range(rhs)])
    return pool


def rbytes(g):
    return 100 * g.n3


def requests(seq, tols=(1e-8, 1e-10)):
    return [Request(k, gid, k % 2, tols[k % 2], 0.0001 * k) for k, gid in enumerate(seq)]


@pytest.mark.parametrize("Eng", ENGINES)
def test_every_request_served_and_grid_order_kept(Eng):
    pool = fake_pool([100, 200, 300, 400, 500])
    eng = Eng(10_000)
    srv = Server(pool, eng, 1e12, rbytes, chunk=8, keep_q=False)
    rng = np.random.default_rng(0)
    reqs = requests(rng.integers(0, 5, 60))
    srv.run(reqs, realtime=False)
    assert all(r.t_done >= 0 and r.status == 0 for r in reqs)
    for gid in range(5):
        chain = [r for r in reqs if r.grid == gid]
        for a, b in zip(chain, chain[1:]):
            assert b.t_admit >= a.t_done  # one in flight per grid, in arrival order
        # the first request on a grid is cold, later ones warm-start
        assert not chain[0].warm and chain[0].iters == FakeEngine._iters(chain[0].tol, False)
        assert all(r.warm and r.iters == FakeEngine._iters(r.tol, True) for r in chain[1:])
    assert srv.evictions == 0
    assert srv.work == sum(r.iters * r.unknowns for r in reqs)


@pytest.mark.parametrize("Eng", ENGINES)
def test_requests_join_running_launches(Eng):
    """Continuous batching: requests admitted together share their launches."""
    pool = fake_pool([100, 100, 100])
    srv = Server(pool, Eng(10_000), 1e12, rbytes, chunk=4, keep_q=False)
    reqs = requests([0, 1, 2])
    srv.run(reqs, realtime=False)
    # 40 iterations at 1e-8 (requests 0, 2) and 80 at 1e-10 (request 1) in chunks of 4
    assert [r.launch_done for r in reqs] == [10, 20, 10]
    assert srv.launches == 20


@pytest.mark.parametrize("Eng", ENGINES)
def test_budget_admission_and_lru_eviction(Eng):
    pool = fake_pool([1000, 1000, 1000, 1000])
    eng = Eng(10_000)
    budget = 2.5 * 100 * 1000  # room for two grids
    srv = Server(pool, eng, budget, rbytes, chunk=8, keep_q=False)
    reqs = requests([0, 1, 2, 3, 0, 1, 2, 3, 0])
    srv.run(reqs, realtime=False)
    assert all(r.t_done >= 0 for r in reqs)
    assert eng.peak <= 2000
    assert srv.evictions >= 5
    assert srv.used <= budget
    assert not any(r.warm for r in reqs[4:8])  # each revisit found its grid evicted


@pytest.mark.parametrize("Eng", ENGINES)
def test_engine_capacity_triggers_eviction(Eng):
    pool = fake_pool([600, 600, 600])
    eng = Eng(1300)  # the arena holds two grids although the budget holds all
    srv = Server(pool, eng, 1e12, rbytes, chunk=8, keep_q=False)
    reqs = requests([0, 1, 2, 0])
    srv.run(reqs, realtime=False)
    assert all(r.t_done >= 0 for r in reqs)
    assert srv.evictions >= 1 and eng.peak <= 1300


def test_grid_over_budget_raises():
    srv = Server(fake_pool([1000]), FakeEngine(10_000), 1000.0, rbytes, keep_q=False)
    with pytest.raises(SolverError):
        srv.run(requests([0]), realtime=False)


def test_request_right_hand_side_mix():
    pool = fake_pool([10], rhs=2)
    r = Request(0, 0, 1, 1e-8, 0.0, mix=0.25)
    assert np.allclose(request_src(pool, r), 0.75 * 2.0 + 0.25 * 1.0)
    assert request_src(pool, Request(1, 0, 0, 1e-8, 0.0)) is pool[0][0].src


@pytest.mark.parametrize("Eng", ENGINES)
def test_poisson_stream_and_realtime_loop(Eng):
    reqs = poisson_stream(3, 2, rate=2000.0, seconds=0.05, seed=3)
    n = len(reqs)
    assert abs(n - 100) < 5 * np.sqrt(100)
    t = [r.t_arrival for r in reqs]
    assert t == sorted(t) and t[-1] < 0.05
    assert {r.tol for r in reqs} <= {1e-8, 1e-10}
    assert all(0.0 <= r.mix < 1.0 for r in reqs)
    srv = Server(fake_pool([100, 100, 100]), Eng(10_000), 1e12, rbytes, chunk=16, keep_q=False)
    srv.run(reqs, realtime=True)
    assert all(r.t_done >= r.t_arrival and r.t_admit >= r.t_arrival for r in reqs)
    rep = latency_report(reqs, srv.t_end)
    assert rep["completed"] == n and rep["p99_ms"] >= rep["p50_ms"] > 0
    assert rep["status_counts"] == {0: n}
    tail = rep["tail"]
    assert tail["requests"] >= 1 and 0 <= tail["behind_same_grid"] <= tail["requests"]
    assert tail["mean_admission_wait_ms"] >= 0 and tail["mean_solve_ms"] >= 0


def test_tail_report_counts_requests_behind_their_grid():
    """A request arriving while an earlier request on its grid is unfinished is
    counted as waiting behind its grid."""
    from suntans_gb300.serve import tail_report
    a = Request(0, 0, 0, 1e-8, 0.0, t_admit=0.0, t_done=1.0, unknowns=10, iters=5)
    b = Request(1, 0, 1, 1e-8, 0.5, t_admit=1.0, t_done=2.0, unknowns=10, iters=5)  # behind a
    c = Request(2, 1, 0, 1e-8, 0.0, t_admit=0.0, t_done=0.1, unknowns=10, iters=5)
    t = tail_report([a, b, c], 1000.0)
    assert t["requests"] == 2 and t["behind_same_grid"] == 1 and t["distinct_grids"] == 1
    assert abs(t["mean_admission_wait_ms"] - 250.0) < 1e-9


def test_prefetched_sources_equal_direct():
    pool = fake_pool([10, 20], rhs=3)
    reqs = poisson_stream(2, 3, rate=1000.0, seconds=0.2, seed=5)
    pre = PrefetchedSources(pool, reqs, workers=2, depth=8)
    try:
        for r in reqs:
            assert np.array_equal(pre.get(r), request_src(pool, r))
    finally:
        pre.close()
    srv = Server(pool, FakeEngine(10_000), 1e12, rbytes, chunk=16, keep_q=False,
                 sources=PrefetchedSources(pool, reqs).get)
    srv.run(reqs, realtime=False)
    assert all(r.t_done >= 0 for r in reqs)


def test_overlapped_loop_admits_during_launches():
    """With launch / wait, a request arriving while a launch runs is admitted
    before that launch is waited for and joins the next one."""
    pool = fake_pool([100, 100])
    eng = FakeAsyncEngine(10_000)
    srv = Server(pool, eng, 1e12, rbytes, chunk=4, keep_q=False)
    reqs = requests([0, 1])
    seen = []
    orig_wait = eng.wait

    def wait():
        seen.append(sorted(eng.inst))  # problems resident when the launch in flight is waited for
        return orig_wait()

    eng.wait = wait
    srv.run(reqs, realtime=False)
    assert all(r.t_done >= 0 for r in reqs)
    assert srv.launches == 20 and srv.work == sum(r.iters * r.unknowns for r in reqs)
    assert seen[0] == [0, 1]


@pytest.mark.parametrize("Eng", ENGINES)
def test_copies_serve_a_hot_grid_in_parallel(Eng):
    """With copies = 2, three requests on one grid arriving together: the first
    two run at once on two resident copies (the second cold), the third waits
    for an idle copy and warm-starts there; with copies = 1 they run one after
    another.  Copies count against the budget like any resident grid."""
    pool = fake_pool([100, 100])
    for copies, launches_max in ((1, 3 * 5), (2, 2 * 5)):
        eng = Eng(10_000)
        srv = Server(pool, eng, 1e12, rbytes, chunk=8, keep_q=False, copies=copies)
        reqs = [Request(k, 0, k % 2, 1e-8, 0.0) for k in range(3)]
        srv.run(reqs, realtime=False)
        assert all(r.t_done >= 0 and r.iters > 0 for r in reqs)
        assert srv.ncopy[0] == copies and srv.used == copies * rbytes(pool[0][0].grid)
        assert [r.warm for r in reqs] == ([False, True, True] if copies == 1 else [False, False, True])
        assert srv.launches <= launches_max
    # budget for one copy only: the second copy is not created, nothing is evicted
    eng = FakeEngine(10_000)
    srv = Server(pool, eng, 1.5 * rbytes(pool[0][0].grid), rbytes, chunk=8, keep_q=False, copies=2)
    reqs = [Request(k, 0, 0, 1e-8, 0.0) for k in range(2)]
    srv.run(reqs, realtime=False)
    assert srv.ncopy[0] == 1 and srv.evictions == 0 and all(r.t_done >= 0 for r in reqs)


class StridedEngine(FakeEngine):
    """FakeEngine whose launches honour per-problem strides (a problem with
    stride s advances on every s-th global iteration of a launch)."""

    def __init__(self, cap):
        super().__init__(cap)
        self.strides = {}
        self.log = []

    def set_stride(self, i, s):
        self.strides[i] = s
        self.log.append((i, s))

    def run(self, max_iters=0):
        work, running = 0, 0
        for i, I in self.inst.items():
            if I["state"] in (1, 2):
                s = self.strides.get(i, 1)
                cap = I["left"] if max_iters <= 0 else -(-max_iters // s)
                k = min(I["left"], cap)
                I["left"] -= k
                I["it"] += k
                work += k * I["n"]
                I["state"] = 3 if I["left"] == 0 else 2
                running += I["state"] != 3
        return running, 0.1, work

    def release(self, i):
        super().release(i)
        self.strides.pop(i, None)


def test_strides_slow_large_problems_while_small_ones_are_in_flight():
    """stride_cap 4, ratio 8: beside a 100-unknown problem, one of 1000 gets
    stride 2 and one of 5000 stride 4; alone, a large problem runs at stride 1
    again; with the default stride_cap nothing is set."""
    pool = fake_pool([100, 1000, 5000], rhs=1)
    eng = StridedEngine(10 ** 9)
    srv = Server(pool, eng, 1e12, rbytes, chunk=8, keep_q=False, stride_cap=4, stride_ratio=8.0)
    reqs = [Request(k, k, 0, 1e-10, 0.0) for k in range(3)]
    srv.run(reqs, realtime=False)
    first = dict(eng.log[:2])
    assert first == {1: 2, 2: 4}, eng.log
    # once the small request is done the large ones go back to stride 1
    assert (1, 1) in eng.log[2:] or (2, 1) in eng.log[2:], eng.log
    assert all(r.t_done >= 0 and r.iters == 80 for r in reqs)
    # 80 iterations at chunk 8: the small request in launch 10; beside it the
    # others advanced 40 (stride 2) and 20 (stride 4), then 8 per launch
    assert [r.launch_done for r in reqs] == [10, 15, 18]
    eng2 = StridedEngine(10 ** 9)
    Server(pool, eng2, 1e12, rbytes, chunk=8, keep_q=False).run([Request(k, k, 0, 1e-10, 0.0) for k in range(3)],
                                                                  realtime=False)
    assert eng2.log == []
