"""Replicas across ranks: the solvers do not shard, so N GPUs run N independent
replicas (bench.py --gpus N) with no data-path collective; only the bench's
barrier and max-over-ranks timing cross ranks.  Checked here with the gloo
backend on CPU at world size 2: each rank builds the same seeded workload,
solves its own share of independent problems with the oracle, and the
reductions the bench uses (max of times, sum of work) combine them."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _problems():
    from suntans_gb300 import gridgen as gg
    g = gg.quad_channel(8, 4, Nkmax=6, seed=1)
    return g, [gg.make_q_problem(g, seed=s) for s in range(4)]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    from oracle.oracle import Oracle
    from suntans_gb300.grid import SolverProps
    g, probs = _problems()
    o = Oracle("port")
    pr = SolverProps(qprecond=1, qmaxiters=500, qepsilon=1e-10)
    work, sums = 0, []
    for p in probs[rank::world]:  # independent problems, no exchange
        q, n = o.cgsolveq(p, pr)
        work += g.n_q() * n
        sums.append(float(np.abs(q).sum()))
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(work)])
    dist.all_reduce(w)
    out[rank] = (float(t.item()), float(w.item()), sums)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0  # max over ranks
    assert res[0][1] == res[1][1] > 0     # whole-job work
    # each replica's results equal a single-process solve of the same problems
    from oracle.oracle import Oracle
    from suntans_gb300.grid import SolverProps
    g, probs = _problems()
    o = Oracle("port")
    pr = SolverProps(qprecond=1, qmaxiters=500, qepsilon=1e-10)
    solo = [float(np.abs(o.cgsolveq(p, pr)[0]).sum()) for p in probs]
    assert res[0][2] == solo[0::2] and res[1][2] == solo[1::2]
