"""Launch-shape autotuner of the batched pressure solver.

The batched kernel's shape has two runtime knobs:

* CTAs per SM (1..3 resident at the kernel's register budget): more CTAs hide
  the latency of the face gathers, fewer make the per-iteration grid barrier
  cheaper;
* storage slots per tile (the unit of work a CTA's eight compute warps take at
  once; with the 1024-slot maximum a warp owns 128 slots, i.e. several columns
  of a 10..60-level grid).  Small tiles spread a batch of small problems over
  more CTAs; large tiles amortise the tile header and the pipeline hand-offs.

`autotune` measures unknown-iterations per second for every pair on the
caller's own problems (a short run of `iters` iterations after the set-up
phase, every instance active) and returns the fastest.  A pair whose tile
count exceeds what that many CTAs can list is recorded as infeasible.  The
pipeline depth and the fusion of the CG steps into two passes per iteration
are fixed in the kernel; they are not swept.
"""
from __future__ import annotations

import numpy as np

from .batch import Batch, capacity_for
from .capi import OOM, SolverError

CTAS_PER_SM = (1, 2, 3)
TILE_SLOTS = (256, 512, 1024)


def sm_count(device=0) -> int:
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


def autotune(problems, qprecond=1, tol=1e-10, maxiters=20000, iters=12, ctas_per_sm=CTAS_PER_SM,
             tile_slots=TILE_SLOTS, device=0, sample=None):
    """Returns (best, table): best = {"ctas_per_sm", "tile_slots", "rate", "ms"}; table lists every candidate.

    problems: QProblem list (all share maxfaces).  sample: use at most this many
    problems (evenly spaced after sorting by size), None = all."""
    probs = list(problems)
    if sample is not None and len(probs) > sample:
        order = np.argsort([p.grid.n3 for p in probs])
        probs = [probs[i] for i in order[np.linspace(0, len(probs) - 1, sample).astype(int)]]
    F = probs[0].grid.maxfaces
    nsm = sm_count(device)
    table = []
    for ts in tile_slots:
        b = Batch(qprecond=qprecond, maxfaces=F, device=device, **capacity_for([p.grid for p in probs]))
        try:
            b.set_tile_slots(ts)
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
                    table.append({"ctas_per_sm": cps, "tile_slots": ts, "rate": 0.0, "ms": None,
                                  "infeasible": str(e)})
                    continue
                table.append({"ctas_per_sm": cps, "tile_slots": ts, "rate": work / (ms / 1e3) if ms > 0 else 0.0,
                              "ms": ms})
        finally:
            b.close()
    best = max(table, key=lambda r: r["rate"])
    return dict(best), table
