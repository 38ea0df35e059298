"""Serving loop for pressure solves: continuous batching over the batched solver.

Requests (grid, right-hand side, tolerance) arrive over time.  Every grid a
request names becomes a resident problem of one `Batch`: its connectivity,
coefficients and last solution stay in HBM, and the next request on the same
grid only uploads its right-hand side and starts from that solution (the warm
start the model itself uses: CGSolveQ begins from the previous phys->qc,
main/phys.c:2411-2550).  The device runs one persistent launch of at most
`chunk` CG iterations over every active problem; between launches the host
harvests finished problems and admits requests that arrived meanwhile, so new
work joins the running batch at the next launch instead of waiting for it to
drain.

Admission is by HBM budget: a grid becomes resident only while the bytes of
all resident grids (`request_bytes`) stay within the budget and the batch's
arenas have room; otherwise idle resident grids are evicted least recently
used first, and when nothing is evictable the request waits.  Requests on one
grid run one at a time in arrival order, so the warm-start chain of a grid
does not depend on what else is in flight: a result is the same alone and in
any mix (the batched kernel is composition-independent bit for bit).

A request's right-hand side is (1 - mix) x rhs_j + mix x rhs_(j+1) of its
grid's stored right-hand sides.  With the reference's relative stopping rule
(sqrt(eps/eps0) < tol, eps0 from the initial guess) a warm start from the
solution of the very same right-hand side would ask for a residual below
round-off, so streams draw mix per request.

The engine is duck-typed (`Batch` or a host fake with the same methods), so
the scheduling logic is testable without a GPU.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np

from .capi import OOM, SolverError


@dataclasses.dataclass
class Request:
    rid: int
    grid: int            # index into the grid pool
    rhs: int             # index of the right-hand side among the grid's problems
    tol: float
    t_arrival: float     # seconds from the start of the stream
    mix: float = 0.0     # weight of the next stored right-hand side
    t_admit: float = -1.0
    t_done: float = -1.0
    iters: int = 0
    status: int = -1
    unknowns: int = 0
    launch_done: int = -1  # serving-loop launch after which the result was harvested
    warm: bool = False     # started from the grid's resident previous solution
    copy: int = -1         # the resident copy of the grid that served it
    warm_from: int = -1    # rid of the request whose solution was its initial guess (-1: cold)
    q: np.ndarray | None = None


def poisson_stream(n_grids, rhs_per_grid, rate, seconds, seed=7, tols=(1e-8, 1e-10)):
    """Open-loop Poisson arrivals: exponential gaps at `rate`/s for `seconds`,
    each request a uniformly drawn (grid, right-hand side, mix, tolerance)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        out.append(Request(len(out), int(rng.integers(n_grids)), int(rng.integers(rhs_per_grid)),
                           float(tols[int(rng.integers(len(tols)))]), t, mix=float(rng.uniform())))
    return out


def request_src(pool, r: Request):
    probs = pool[r.grid]
    p = probs[r.rhs]
    if r.mix == 0.0 or len(probs) < 2:
        return p.src
    o = probs[(r.rhs + 1) % len(probs)]
    return (1.0 - r.mix) * p.src + r.mix * o.src


class PrefetchedSources:
    """Right-hand sides of a request stream prepared ahead of arrival by worker
    threads (the stream's clients), so that producing them is not part of the
    server's critical path.  `get(r)` returns request r's array; at most
    `depth` requests beyond the latest one asked for are prepared."""

    def __init__(self, pool, reqs, workers=2, depth=64):
        import concurrent.futures as cf
        self.pool, self.depth = pool, depth
        self.reqs = sorted(reqs, key=lambda r: r.t_arrival)
        self.pos = {r.rid: k for k, r in enumerate(self.reqs)}
        self.ex = cf.ThreadPoolExecutor(workers)
        self.fut = {}
        self.next = 0
        self._fill(0)

    def _fill(self, upto):
        while self.next < len(self.reqs) and self.next <= upto + self.depth:
            r = self.reqs[self.next]
            self.fut[r.rid] = self.ex.submit(request_src, self.pool, r)
            self.next += 1

    def get(self, r):
        self._fill(self.pos.get(r.rid, 0))
        f = self.fut.pop(r.rid, None)
        return f.result() if f is not None else request_src(self.pool, r)

    def close(self):
        self.ex.shutdown(wait=False, cancel_futures=True)


class Server:
    """pool[g] is a list of QProblem on grid g (its stored right-hand sides).
    sources: callable request -> right-hand side (default: request_src).

    copies: resident copies a grid may have.  With 1 (the default) a grid's
    requests are served one at a time in arrival order, each warm-started from
    the previous one's solution, so every result is the same bits alone or in
    any mix.  The tail of the request stream comes from that queue (a hot
    grid's requests wait behind one another; `tail_report`).  With copies > 1
    a request arriving while its grid is busy goes to an idle copy of the grid
    (warm-started from that copy's last solution) or, budget allowing, to a
    new copy, warm-started from the grid's latest finished solution (cold when
    it has none): the queue goes, and each result is still a solve of its own
    request to its tolerance from the initial guess it was given
    (Request.warm_from) -- the same within the tolerance, not the same bits,
    as when served alone."""

    def __init__(self, pool, engine, budget_bytes, request_bytes, chunk=64, maxiters=20000, keep_q=True,
                 clock=time.perf_counter, sources=None, copies=1, stride_cap=1, stride_ratio=8.0):
        self.pool = pool
        self.engine = engine
        self.budget = float(budget_bytes)
        self.rbytes = [int(request_bytes(p[0].grid)) for p in pool]
        self.chunk = int(chunk)
        self.maxiters = int(maxiters)
        self.keep_q = keep_q
        self.clock = clock
        self.copies = max(1, int(copies))
        self.resident = collections.OrderedDict()  # (grid, copy) -> instance id (LRU order)
        self.busy = {}                             # (grid, copy) -> Request in flight
        self.ncopy = collections.Counter()         # grid -> resident copies
        self.copy_last = {}                        # (grid, copy) -> rid of its last finished request
        self.grid_last = {}                        # grid -> (rid, solution) of its latest finished request
        self.used = 0
        self.evictions = 0
        self.launches = 0
        self.resubmits = 0
        self.work = 0
        self.device_ms = 0.0
        self.t0 = self.clock()
        self.sources = sources or (lambda r: request_src(pool, r))
        self.qbuf = {}  # grid -> reusable result buffer when results are not kept
        # size-aware sharing of the lockstep launches (_set_strides)
        self.stride_cap = max(1, int(stride_cap))
        self.stride_ratio = float(stride_ratio)
        self.stride_of = {}  # instance id -> stride last set
        self.host_s = {"admit": 0.0, "launch": 0.0, "harvest": 0.0}  # wall time by loop part

    # -- admission --------------------------------------------------------
    def _evict_one(self, avoid) -> bool:
        for key, iid in self.resident.items():
            if key not in self.busy and key[0] != avoid:
                self.engine.release(iid)
                self.stride_of.pop(iid, None)  # the id may be reused by a later add (stride 1)
                del self.resident[key]
                self.ncopy[key[0]] -= 1
                self.used -= self.rbytes[key[0]]
                self.evictions += 1
                return True
        return False

    def _busy_grids(self):
        return {key[0] for key in self.busy}

    def _admit(self, r: Request) -> bool:
        g = r.grid
        idle = [key for key in self.resident if key[0] == g and key not in self.busy]
        if idle:
            key = idle[-1]  # the most recently used copy
            iid = self.resident.pop(key)
            self.resident[key] = iid
            self.engine.resubmit(iid, self.sources(r), tol=r.tol, maxiters=self.maxiters, warm=True)
            self.resubmits += 1
            r.warm = True
            r.warm_from = self.copy_last.get(key, -1)
        else:
            if self.ncopy[g] >= self.copies:
                return False
            if self.rbytes[g] > self.budget:
                raise SolverError(OOM, f"grid {g} needs {self.rbytes[g]} bytes, budget {self.budget:.0f}")
            while self.used + self.rbytes[g] > self.budget:
                if not self._evict_one(g):
                    return False
            prob = self.pool[g][r.rhs]
            if r.mix != 0.0:
                prob = type(prob)(**{**prob.__dict__, "src": self.sources(r)})
            last = self.grid_last.get(g) if self.copies > 1 else None
            if last is not None:
                # a further copy of a grid in use starts from its latest solution
                prob = type(prob)(**{**prob.__dict__, "q": last[1]})
            while True:
                try:
                    iid = self.engine.add(prob, tol=r.tol, maxiters=self.maxiters)
                    break
                except SolverError as e:
                    if e.code != OOM:
                        raise
                    if not self._evict_one(g):
                        return False
            c = 0
            while (g, c) in self.resident:
                c += 1
            key = (g, c)
            if last is not None:
                r.warm = True
                r.warm_from = last[0]
            self.resident[key] = iid
            self.ncopy[g] += 1
            self.used += self.rbytes[g]
        self.busy[key] = r
        r.copy = key[1]
        r.t_admit = self.clock() - self.t0
        return True

    def _harvest(self, only=None):
        for key, r in list(self.busy.items()):
            g = key[0]
            if only is not None and g not in only:
                continue
            iid = self.resident[key]
            if self.engine.state(iid) == 3:  # INST_DONE
                if self.keep_q:
                    q, st = self.engine.result(iid, self.pool[g][r.rhs].q, release=False)
                else:
                    if g not in self.qbuf:
                        self.qbuf[g] = np.zeros(self.pool[g][0].grid.n3)
                    q, st = self.engine.result(iid, None, release=False, out=self.qbuf[g])
                r.t_done = self.clock() - self.t0
                r.launch_done = self.launches
                r.iters, r.status, r.unknowns = int(st.niters), int(st.status), int(st.unknowns)
                if self.keep_q:
                    r.q = q
                self.copy_last[key] = r.rid
                if self.copies > 1:
                    self.grid_last[g] = (r.rid, q if self.keep_q else self.qbuf[g])
                del self.busy[key]

    def _set_strides(self):
        """Every global iteration of a launch costs time in proportion to the
        unknowns of the problems taking part, so in lockstep a small request
        pays for the large ones beside it.  With stride_cap > 1 a problem in
        flight with at least stride_ratio x s times the storage of the
        smallest one in flight advances only on every s-th global iteration
        (s = 2, 4, ... up to stride_cap): small requests finish sooner, large
        ones later, and no result changes (the engine's strides leave every
        problem's own iterates alone)."""
        if self.stride_cap <= 1 or not hasattr(self.engine, "set_stride"):
            return
        sizes = {key: self.pool[key[0]][0].grid.n3 for key in self.busy}  # storage slots
        if not sizes:
            return
        smallest = min(sizes.values())
        for key, n in sizes.items():
            s = 1
            while s < self.stride_cap and n >= self.stride_ratio * smallest * s:
                s *= 2
            iid = self.resident[key]
            if self.stride_of.get(iid, 1) != s:
                self.engine.set_stride(iid, s)
                self.stride_of[iid] = s

    def _admit_waiting(self, queues):
        """Admits waiting requests, oldest first across grids; a grid takes as
        many of its waiting requests as it has idle or new copies (one at a
        time with copies = 1: a grid's later requests wait for its earlier
        ones).  Returns how many."""
        n = 0
        heads = sorted((q[0].t_arrival, g) for g, q in queues.items() if q)
        for _, g in heads:
            while queues.get(g) and self._admit(queues[g][0]):
                queues[g].popleft()
                n += 1
            if g in queues and not queues[g]:
                del queues[g]
        return n

    # -- the loop -----------------------------------------------------------
    def run(self, requests, realtime=True, drain_limit=None):
        """Serves `requests` (sorted by t_arrival).  realtime=False admits every
        request at once (arrival times ignored).  drain_limit (s) stops the loop
        with requests unfinished.  Returns the requests.

        With an engine that can launch and wait separately, the host reads back
        the problems the previous launch finished while the next launch runs,
        except those whose grid has a request waiting: those are read back and
        the waiting request admitted before the launch, so that a grid's
        requests follow one another launch by launch as in the serial loop."""
        if hasattr(self.engine, "launch") and hasattr(self.engine, "wait"):
            return self._run_overlapped(requests, realtime, drain_limit)
        reqs = sorted(requests, key=lambda r: r.t_arrival)
        queues = collections.OrderedDict()  # grid -> deque of waiting requests, in arrival order
        npending = 0
        self.t0 = self.clock()
        i = 0
        while True:
            now = self.clock() - self.t0
            while i < len(reqs) and (not realtime or reqs[i].t_arrival <= now):
                queues.setdefault(reqs[i].grid, collections.deque()).append(reqs[i])
                npending += 1
                i += 1
            # admit waiting requests, oldest first (_admit_waiting)
            t1 = self.clock()
            npending -= self._admit_waiting(queues)
            t2 = self.clock()
            self.host_s["admit"] += t2 - t1
            if self.busy:
                self._set_strides()
                _, ms, work = self.engine.run(max_iters=self.chunk)
                t3 = self.clock()
                self.launches += 1
                self.work += work
                self.device_ms += ms
                self._harvest()
                self.host_s["launch"] += t3 - t2
                self.host_s["harvest"] += self.clock() - t3
            elif npending:
                raise RuntimeError("requests pending with nothing running: budget too small")
            elif i < len(reqs):
                wait = reqs[i].t_arrival - (self.clock() - self.t0)
                if wait > 0:
                    time.sleep(min(wait, 0.001))
            else:
                break
            if drain_limit is not None and self.clock() - self.t0 > drain_limit:
                break
        self.t_end = self.clock() - self.t0
        return reqs


    def _run_overlapped(self, requests, realtime, drain_limit):
        reqs = sorted(requests, key=lambda r: r.t_arrival)
        queues = collections.OrderedDict()
        npending = 0
        self.t0 = self.clock()
        i = 0
        inflight = False
        while True:
            now = self.clock() - self.t0
            while i < len(reqs) and (not realtime or reqs[i].t_arrival <= now):
                queues.setdefault(reqs[i].grid, collections.deque()).append(reqs[i])
                npending += 1
                i += 1
            t1 = self.clock()
            if inflight:
                _, ms, work = self.engine.wait()
                inflight = False
                if ms > 0 or work > 0:
                    self.launches += 1
                self.work += work
                self.device_ms += ms
            t2 = self.clock()
            self.host_s["launch"] += t2 - t1
            # grids with a request waiting: read back now, so that request joins the next launch
            self._harvest(only={g for g, q in queues.items() if q})
            t3 = self.clock()
            self.host_s["harvest"] += t3 - t2
            npending -= self._admit_waiting(queues)
            t4 = self.clock()
            self.host_s["admit"] += t4 - t3
            if self.busy:
                self._set_strides()
                self.engine.launch(max_iters=self.chunk)
                inflight = True
                # the other finished problems are read back while this launch runs
                self._harvest()
                self.host_s["harvest"] += self.clock() - t4
            elif npending:
                raise RuntimeError("requests pending with nothing running: budget too small")
            elif i < len(reqs):
                wait = reqs[i].t_arrival - (self.clock() - self.t0)
                if wait > 0:
                    time.sleep(min(wait, 0.001))
            else:
                break
            if drain_limit is not None and self.clock() - self.t0 > drain_limit:
                break
        if inflight:
            _, ms, work = self.engine.wait()
            self.work += work
            self.device_ms += ms
            self._harvest()
        self.t_end = self.clock() - self.t0
        return reqs


def latency_report(reqs, t_end):
    """p50/p99 latency (arrival to harvest) over completed requests, throughput over the run."""
    done = [r for r in reqs if r.t_done >= 0]
    lat = np.array([r.t_done - r.t_arrival for r in done]) * 1e3
    out = {"requests": len(reqs), "completed": len(done),
           "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
           "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
           "mean_ms": float(lat.mean()) if len(lat) else None,
           "makespan_s": t_end,
           "unknown_iters": int(sum(r.unknowns * r.iters for r in done)),
           "status_counts": {int(s): int(sum(r.status == s for r in done)) for s in sorted({r.status for r in done})},
           "mean_iters": float(np.mean([r.iters for r in done])) if done else None,
           "mean_unknowns": float(np.mean([r.unknowns for r in done])) if done else None}
    out["unknown_iters_per_s"] = out["unknown_iters"] / t_end if t_end > 0 else 0.0
    out["served_per_s"] = len(done) / t_end if t_end > 0 else 0.0
    out["tail"] = tail_report(reqs, out["p99_ms"])
    return out


def tail_report(reqs, p99_ms):
    """Where the slowest requests (latency >= p99) spent their time, request by
    request: waiting for admission (arrival to admission) against being solved
    (admission to harvest), how many of them were admitted only when the
    previous request on the same grid had finished (requests on one grid are
    served one at a time), and their share of the grids and sizes."""
    done = [r for r in reqs if r.t_done >= 0]
    if not done or p99_ms is None:
        return None
    prev_done = {}
    behind = {}
    for r in sorted(reqs, key=lambda x: x.t_arrival):
        pd = prev_done.get(r.grid)
        behind[r.rid] = pd is not None and (pd < 0 or pd > r.t_arrival)
        prev_done[r.grid] = r.t_done
    slow = [r for r in done if (r.t_done - r.t_arrival) * 1e3 >= p99_ms]
    if not slow:
        return None
    wait = np.array([max(r.t_admit - r.t_arrival, 0.0) for r in slow]) * 1e3
    serve = np.array([r.t_done - max(r.t_admit, r.t_arrival) for r in slow]) * 1e3
    grids = {}
    for r in slow:
        grids[r.grid] = grids.get(r.grid, 0) + 1
    return {"requests": len(slow),
            "mean_admission_wait_ms": float(wait.mean()), "mean_solve_ms": float(serve.mean()),
            "behind_same_grid": int(sum(behind[r.rid] for r in slow)),
            "distinct_grids": len(grids), "top_grid_share": max(grids.values()) / len(slow),
            "mean_unknowns": float(np.mean([r.unknowns for r in slow])),
            "mean_iters": float(np.mean([r.iters for r in slow]))}
