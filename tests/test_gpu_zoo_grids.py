"""The FP64 device solvers on grids the reference ships with its examples
(the riverplume hexagon grid, cells of 5-7 faces, and its hybrid triangle /
quad grid with maxFaces 7), against the reference's own solutions stored in
tests/golden/examples/ (make_example_golden.py): relative L2 <= 1e-9 over the
active levels and iteration counts within the summation-order allowance."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300.capi import Context, OK
from tests._cases import rel_l2, stopping_ratio
from tests._golden import example_names, load_example, props_for
from tests.test_gpu_parity import TOL, iters_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", example_names())
def test_example_grid_cgsolveq(gpu_lib, name):
    """The solution is checked first (relative L2 against the reference's, and
    the reference's stopping ratio re-evaluated on it), then the iteration
    count against the span of the oracle's sequential and pairwise counts."""
    g, qp, hp, props, d = load_example(name)
    m = g.active_mask()
    o = Oracle("port")
    ctx = Context(g)
    for qpc in (0, 1, 2):
        pr = props_for(props, qprecond=qpc)
        q, st = ctx.cgsolveq(qp, pr)
        assert st.status == OK
        assert rel_l2(q, d[f"q_qp{qpc}"], m) <= TOL, qpc
        assert stopping_ratio(o, qp, q, qpc) < 10 * pr.qepsilon, qpc
        n_seq, n_pair = o.iteration_span(qp, pr)
        assert n_seq == int(d[f"n_qp{qpc}"])
        assert iters_close(st.niters, n_seq, n_pair), (qpc, st.niters, n_seq, n_pair)
    ctx.close()


@pytest.mark.parametrize("name", example_names())
def test_example_grid_cgsolve(gpu_lib, name):
    g, qp, hp, props, d = load_example(name)
    comp = g.cellp[g.celldist[0]:g.celldist[1]]
    o = Oracle("port")
    ctx = Context(g)
    for hpc in (0, 1):
        pr = props_for(props, hprecond=hpc)
        h, st = ctx.cgsolve(hp, pr)
        assert st.status == OK
        ref = d[f"h_hp{hpc}"]
        assert np.linalg.norm(h[comp] - ref[comp]) <= TOL * np.linalg.norm(ref[comp]), hpc
        n_seq, n_pair = o.iteration_span(hp, pr, solver="h")
        assert iters_close(st.niters, n_seq, n_pair), (hpc, st.niters, n_seq, n_pair)
    ctx.close()
