"""The device solvers on the solves of a 10-step run of the reference model on
the 64 x 16 lock-exchange channel (tests/golden/runs/lockexchange_cfg1.npz, written
by make_lockexchange_golden.py from the reference's own CGSolveQ / CGSolve
calls): through the C ABI, each solve's recorded inputs give the reference's
solution within relative L2 1e-9, with the iteration count within the
summation-order allowance; the batched mixed-precision solver meets the same
bound on the pressure solves."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300.batch import Batch, capacity_for
from suntans_gb300.capi import Context, OK
from tests._cases import rel_l2
from tests._golden import load_lockexchange
from tests.test_gpu_parity import TOL, iters_close

pytestmark = pytest.mark.gpu


def test_lockexchange_cgsolveq_steps(gpu_lib):
    d, props, grid_at, q_problem, h_problem = load_lockexchange()
    o = Oracle("port")
    for s in d["q_steps"]:
        p, ref, n = q_problem(int(s))
        m = p.grid.active_mask()
        ctx = Context(p.grid)
        q, st = ctx.cgsolveq(p, props)
        ctx.close()
        assert st.status == OK
        assert rel_l2(q, ref, m) <= TOL, s
        assert np.array_equal(q[~m], p.q[~m])
        assert iters_close(st.niters, *o.iteration_span(p, props)), (s, st.niters, n)


def test_lockexchange_cgsolve_steps(gpu_lib):
    d, props, grid_at, q_problem, h_problem = load_lockexchange()
    o = Oracle("port")
    g = grid_at(1)
    comp = g.comp_cells()
    ctx = Context(g)
    for s in d["h_steps"]:
        p, ref, n = h_problem(int(s))
        h, st = ctx.cgsolve(p, props)
        assert st.status == OK
        assert np.linalg.norm(h[comp] - ref[comp]) <= TOL * np.linalg.norm(ref[comp]), s
        assert iters_close(st.niters, *o.iteration_span(p, props, solver="h")), (s, st.niters, n)
    ctx.close()


def test_lockexchange_mixed_pressure_steps(gpu_lib):
    d, props, grid_at, q_problem, h_problem = load_lockexchange()
    for s in d["q_steps"]:
        p, ref, n = q_problem(int(s))
        b = Batch(qprecond=props.qprecond, maxfaces=p.grid.maxfaces, **capacity_for([p.grid]))
        i = b.add(p, tol=props.qepsilon, maxiters=props.qmaxiters)
        b.run()
        q, st = b.result(i, p.q)
        b.close()
        assert st.status == OK
        assert rel_l2(q, ref, p.grid.active_mask()) <= TOL, s
