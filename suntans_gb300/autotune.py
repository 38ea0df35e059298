"""Launch-shape autotuner of the batched pressure solver.

The batched kernel's shape has three runtime knobs:

* CTAs per SM (1..3 resident at the kernel's register budget): more CTAs hide
  the latency of the face gathers, fewer make the per-iteration grid barrier
  cheaper and leave each CTA more shared memory;
* storage slots per tile, i.e. slots per compute lane (256, 512 or 1024
  slots: 1, 2 or 4 slots per lane of the CTA's eight compute warps, each
  warp covering 32, 64 or 128 consecutive levels -- part of a column, or
  several columns of a 10..60-level grid).  Small tiles spread a batch of
  small problems over more CTAs; large tiles amortise the tile header and the
  pipeline hand-offs;
* fusion, the form of an iteration: two passes (operator apply; vector
  update) with the FP32 solution update x += nu p fused into the next apply
  pass, which streams p anyway (13 instead of 14 FP32 values per
  unknown-iteration, a larger pipeline stage), or kept in the update pass --
  the two give the same bits; or one pass per iteration (qprecond 0/1: the
  residual step, the solution update, the new direction and the operator in
  one sweep, the next mu from the sweep's own inner products; 12 values, one
  grid barrier instead of two, a stage of 5 + F streams).

`autotune` measures unknown-iterations per second for every combination on
the caller's own problems (a short run of `iters` iterations after the set-up
phase, every instance active) and returns the fastest.  A combination whose
tile count exceeds what that many CTAs can list is recorded as infeasible.
The pipeline depth (two stages) is fixed in the kernel.
"""
from __future__ import annotations

import numpy as np

from .batch import Batch, capacity_for
from .capi import OOM, SolverError

CTAS_PER_SM = (1, 2, 3)
TILE_SLOTS = (256, 512, 1024)
FUSION = (2, 1, 0)


def sm_count(device=0) -> int:
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


def autotune(problems, qprecond=1, tol=1e-10, maxiters=20000, iters=12, ctas_per_sm=CTAS_PER_SM,
             tile_slots=TILE_SLOTS, fusion=FUSION, device=0, sample=None):
    """Returns (best, table): best = {"ctas_per_sm", "tile_slots", "fusion", "rate", "ms"}; table lists
    every candidate.

    problems: QProblem list (all share maxfaces).  sample: use at most this many
    problems (evenly spaced after sorting by size), None = all."""
    probs = list(problems)
    if sample is not None and len(probs) > sample:
        order = np.argsort([p.grid.n3 for p in probs])
        probs = [probs[i] for i in order[np.linspace(0, len(probs) - 1, sample).astype(int)]]
    F = probs[0].grid.maxfaces
    nsm = sm_count(device)
    table = []
    for ts, fx in [(t, f) for t in tile_slots for f in fusion]:
        b = Batch(qprecond=qprecond, maxfaces=F, device=device, **capacity_for([p.grid for p in probs]))
        try:
            b.set_tile_slots(ts)
            b.set_fusion(fx)
            for p in probs:
                b.add(p, tol=tol, maxiters=maxiters)
            started = False
            for cps in ctas_per_sm:
                b.set(ctas=cps * nsm)
                try:
                    if not started:
                        b.run(max_iters=2)  # set-up phases and the first iterations
                        started = True
                    _, ms, work = b.run(max_iters=iters)
                except SolverError as e:
                    if e.code != OOM:  # more tiles than this CTA count can list: not a candidate
                        raise
                    table.append({"ctas_per_sm": cps, "tile_slots": ts, "fusion": fx, "rate": 0.0,
                                  "ms": None, "infeasible": str(e)})
                    continue
                table.append({"ctas_per_sm": cps, "tile_slots": ts, "fusion": fx,
                              "rate": work / (ms / 1e3) if ms > 0 else 0.0, "ms": ms})
        finally:
            b.close()
    best = max(table, key=lambda r: r["rate"])
    return dict(best), table
