"""Benchmark of the SUNTANS elliptic hot path on GB300.

Workload (default, the plain FP64 method at scale): Delaunay triangulation of
200,000 seeded uniform random points in a 20 km x 10 km rectangle (~400k
triangles), Gaussian seamount (50 m - 30 m exp(-r^2/(2*2000^2))), partial-cell
z-levels Nkmax = 50 stretched 1.02 downward; pressure right-hand side = the
divergence of a seeded N(0, 0.05 m/s) face velocity; free-surface right-hand
side from a seeded N(0, 0.01 m) perturbation.  One step = one CGSolveQ
(qprecond 1) plus one CGSolve (hprecond 1), each to a 1e-10 relative residual,
in FP64.

Metric: unknown-iterations per second = sum over the step's solves of
(unknowns x iterations) / time.  `value` is measured on inputs already
resident in HBM (sgpu_q_solve / sgpu_h_solve) with CUDA events on the solver
stream; `e2e` goes through the drop-in C ABI calls with host jagged arrays
(sgpu_cgsolveq / sgpu_cgsolve), copies included.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cfg2|cfg1] [--qprecond 0|1|2]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

S = 8          # bytes per FP64 value


def q_bytes_per_unknown_iter(qprecond: int, F: int) -> int:
    """Algorithmic HBM bytes per pressure unknown-iteration (FP64).

    apply: read p, one vertical coefficient, F face coefficients, write z
    (3+F values); update: read x, p, r, z, write x, r (6); direction update:
    read r (or M^-1 r), p, write p (3).  qprecond 2 adds the tridiagonal sweep
    (read r, two factor arrays, write M^-1 r) = 3 more values."""
    return S * (12 + F + (3 if qprecond == 2 else 0))


def h_bytes_per_unknown_iter(F: int) -> int:
    """Free surface: apply s(3+F) + 4F bytes of neighbour indices, update 6s, Jacobi + direction 4s."""
    return S * (13 + F) + 4 * F


# ---------------------------------------------------------------------------
def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cfg1"])
    ap.add_argument("--qprecond", type=int, default=1)
    ap.add_argument("--points", type=int, default=200_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    return ap.parse_args()


def make_workload(args):
    from suntans_gb300 import gridgen as gg
    from suntans_gb300.grid import SolverProps
    if args.workload == "cfg1":
        g = gg.quad_channel(64, 16, dx=10.0, dy=10.0, depth=20.0, Nkmax=32, h_sigma=1e-3, seed=1)
        qp = gg.make_q_problem(g, seed=11, sigma_u=0.01, dt=1.0)
        hp = gg.make_h_problem(g, seed=12)
        props = SolverProps(qprecond=args.qprecond, qmaxiters=1000, qepsilon=1e-10, hprecond=1,
                            maxiters=1000, epsilon=1e-10, resnorm=1.0, dt=1.0, theta=0.55)
        desc = {"workload": "quad channel 64x16 cells (dx=dy=10 m), flat 20 m, Nkmax=32, lock-exchange config",
                "cells": g.Nc, "Nkmax": 32}
    else:
        g = gg.delaunay_seamount(args.points, 20_000.0, 10_000.0, Nkmax=50, rstretch=1.02, seed=1,
                                 H0=50.0, amp=30.0, sigma=2000.0, h_sigma=0.01)
        qp = gg.make_q_problem(g, seed=11, sigma_u=0.05, dt=20.0)
        hp = gg.make_h_problem(g, seed=12, sigma_eta=0.01)
        props = SolverProps(qprecond=args.qprecond, qmaxiters=20000, qepsilon=1e-10, hprecond=1,
                            maxiters=20000, epsilon=1e-10, resnorm=1.0, dt=20.0, theta=0.55)
        desc = {"workload": f"Delaunay seamount, {args.points} random points in 20x10 km, Nkmax=50 "
                            f"partial cells rstretch 1.02", "cells": g.Nc, "Nkmax": 50}
    desc.update({"N_q": g.n_q(), "N_h": g.n_h(), "faces": g.maxfaces, "qprecond": args.qprecond, "hprecond": 1,
                 "tolerance": 1e-10, "precision": "fp64"})
    return g, qp, hp, props, desc


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 8:
                for n, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def cpu_baseline(g, qp, hp, props, seconds: float):
    """The oracle port on a bounded sample: CGSolveQ capped at M iterations (plus a full CGSolve)."""
    from oracle.oracle import Oracle
    from suntans_gb300.grid import SolverProps
    o = Oracle("port")
    probe = SolverProps(**{**props.__dict__, "qmaxiters": 2})
    t = time.perf_counter()
    _, n = o.cgsolveq(qp, probe)
    t_probe = time.perf_counter() - t
    per_iter = max(t_probe / max(n, 1), 1e-6)
    m = int(max(2, min(props.qmaxiters, seconds * 0.8 / per_iter)))
    capped = SolverProps(**{**props.__dict__, "qmaxiters": m})
    t = time.perf_counter()
    _, nq = o.cgsolveq(qp, capped)
    tq = time.perf_counter() - t
    work = g.n_q() * nq
    return {"value": work / tq, "unit": "unknown-iters/s", "cores": 1, "kind": "port",
            "sample": f"oracle CGSolveQ (qprecond {props.qprecond}) capped at {nq} iterations on the full "
                      f"N_q={g.n_q()} grid, {tq:.1f} s, 1 thread"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as om
    if not om.available("port"):
        om.build_port()
    g, qp, hp, props, desc = make_workload(args)
    per_step = []
    total_work = 0
    seconds = max(5.0, 60.0 / max(args.steps + args.warmup, 1))
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(g, qp, hp, props, seconds)
        if i >= args.warmup:
            per_step.append(r)
    vals = [r["value"] for r in per_step]
    v = float(np.median(vals))
    line = {"metric": "Poisson CG unknown-iters/s (CGSolveQ+CGSolve, 1e-10 relative residual)", "value": v,
            "unit": "unknown-iters/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": desc, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "unknown-iters/s", "cores": 1, "kind": "port",
                             "sample": per_step[0]["sample"] + "; reference built serial -DNOMPI uses one core"},
            "e2e": {"value": v, "unit": "unknown-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    from suntans_gb300.capi import Context

    g, qp, hp, props, desc = make_workload(args)
    ctx = Context(g, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))

    # ---- device-resident: upload once ----
    ctx.q_upload(qp)
    ctx.h_upload(hp)
    for _ in range(args.warmup):
        ctx.q_solve(props)
        ctx.h_solve(props)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    work = 0
    q_ms, nq, nh = [], [], []
    for _ in range(args.steps):
        sq = ctx.q_solve(props)
        sh = ctx.h_solve(props)
        work += sq.unknowns * sq.niters + sh.unknowns * sh.niters
        q_ms.append(sq.ms_solve)
        nq.append(sq.niters)
        nh.append(sh.niters)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
        w = torch.tensor([float(work)], device="cuda")
        torch.distributed.all_reduce(w)
        work = float(w.item())
    value = work / (ms_total / 1e3)

    # ---- roofline of the dominant kernel (the pressure solve) ----
    bpu = q_bytes_per_unknown_iter(props.qprecond, g.maxfaces)
    q_launch_ms = float(np.mean(q_ms))
    achieved = g.n_q() * float(np.mean(nq)) * bpu / (q_launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()

    # ---- end to end through the drop-in calls with host arrays ----
    e2e_work = 0
    t0 = time.perf_counter()
    h2d = d2h = 0
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        q, sq = ctx.cgsolveq(qp, props)
        h, sh = ctx.cgsolve(hp, props)
        e2e_work += sq.unknowns * sq.niters + sh.unknowns * sh.niters
    e2e_s = time.perf_counter() - t0
    n3, ne3 = g.n3, int(g.Nke.sum())
    h2d = 8 * (4 * n3 + ne3 + g.Ne) + 4 * g.Nc + 8 * (2 * g.Nc + g.Ne)
    d2h = 8 * (n3 + g.Nc)

    line = {"metric": "Poisson CG unknown-iters/s (CGSolveQ+CGSolve, 1e-10 relative residual)", "value": value,
            "unit": "unknown-iters/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded grid and right-hand sides)",
            "config": {**desc, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "not flushed: pressure working set "
                             f"{(13 + g.maxfaces) * 8 * g.n3 / 1e9:.2f} GB > 129 MB L2",
                       "iters_q": int(np.median(nq)), "iters_h": int(np.median(nh))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": f"cgsolveq_kernel<{props.qprecond}>", "bytes_per_unknown_iter": bpu,
                         "peak_kind": peak_kind},
            "e2e": {"value": e2e_work / e2e_s, "unit": "unknown-iters/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": 2 * args.steps, "clocks": clocks}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(g, qp, hp, props, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
