"""The FP64 device solvers on grids the reference ships with its examples
(the riverplume hexagon grid, cells of 5-7 faces, and its hybrid triangle /
quad grid with maxFaces 7), against the reference's own solutions stored in
tests/golden/examples/ (make_example_golden.py): relative L2 <= 1e-9 over the
active levels and iteration counts within the summation-order allowance."""
import numpy as np
import pytest

from suntans_gb300.capi import Context, OK
from tests._cases import rel_l2
from tests._golden import example_names, load_example, props_for
from tests.test_gpu_parity import TOL, iters_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", example_names())
def test_example_grid_cgsolveq(gpu_lib, name):
    g, qp, hp, props, d = load_example(name)
    m = g.active_mask()
    ctx = Context(g)
    for qpc in (0, 1, 2):
        q, st = ctx.cgsolveq(qp, props_for(props, qprecond=qpc))
        assert st.status == OK
        assert iters_close(st.niters, int(d[f"n_qp{qpc}"])), (qpc, st.niters, int(d[f"n_qp{qpc}"]))
        assert rel_l2(q, d[f"q_qp{qpc}"], m) <= TOL, qpc
    ctx.close()


@pytest.mark.parametrize("name", example_names())
def test_example_grid_cgsolve(gpu_lib, name):
    g, qp, hp, props, d = load_example(name)
    comp = g.cellp[g.celldist[0]:g.celldist[1]]
    ctx = Context(g)
    for hpc in (0, 1):
        h, st = ctx.cgsolve(hp, props_for(props, hprecond=hpc))
        assert st.status == OK
        assert iters_close(st.niters, int(d[f"n_hp{hpc}"])), (hpc, st.niters, int(d[f"n_hp{hpc}"]))
        ref = d[f"h_hp{hpc}"]
        assert np.linalg.norm(h[comp] - ref[comp]) <= TOL * np.linalg.norm(ref[comp]), hpc
    ctx.close()
