"""ComputeQSource and Corrector on the device (the steps on either side of
CGSolveQ in Solve, main/phys.c:1273-1287), through the C ABI.

* Both are plain FP64 arithmetic evaluated in the reference's order without
  contraction: the GPU results equal the reference's golden vectors and the
  oracle's outputs bit for bit.
* The fused step (ComputeQSource -> CGSolveQ -> Corrector with the right-hand
  side and the correction kept on the device) matches the oracle's chain of
  the three functions: the correction within relative L2 1e-9 (the solve's
  parity bound) and u, w, q within 1e-8 of the size of the correction they
  received (a max-norm bound on quantities linear in the correction).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.capi import Context, OK
from suntans_gb300.grid import QProblem
from tests._cases import grid_cases, q_props
from tests._golden import fixture_names, load, props_for, step_fields, vgrid_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle():
    return Oracle("port")


@pytest.mark.parametrize("name", fixture_names())
def test_step_functions_match_golden_bitwise(gpu_lib, name):
    g, qp, hp, props, d = load(name)
    st = step_fields(g, d)
    ctx = Context(g)
    ctx.step_grid(st)
    src, D = ctx.compute_qsource(st, props_for(props))
    assert np.array_equal(src, d["qs_src"]) and np.array_equal(D, d["qs_D"])
    u, w, q = ctx.corrector(st, d["q_qp1"], d["qs_D"], props_for(props))
    assert np.array_equal(u, d["corr_u"]) and np.array_equal(w, d["corr_w"]) and np.array_equal(q, d["corr_q"])
    ctx.close()


@pytest.mark.parametrize("gname", [n for n, _ in grid_cases()])
def test_step_functions_match_oracle_bitwise(gpu_lib, oracle, gname):
    g = dict(grid_cases())[gname]()
    if g.normal is None:
        pytest.skip("grid without edge geometry")
    st = gg.make_step_fields(g, seed=41)
    pr = q_props(1)
    ctx = Context(g)
    ctx.step_grid(st)
    src, D = ctx.compute_qsource(st, pr)
    s_ref, D_ref = oracle.compute_qsource(st, pr)
    assert np.array_equal(src, s_ref) and np.array_equal(D, D_ref)
    qc = np.random.default_rng(7).normal(0.0, 0.01, g.n3)
    for a, b in zip(ctx.corrector(st, qc, D_ref, pr), oracle.corrector(st, qc, D_ref, pr)):
        assert np.array_equal(a, b)
    ctx.close()


@pytest.mark.parametrize("qprecond", [0, 1, 2])
@pytest.mark.parametrize("gname", ["tri3000_partial", "quad64x16x32"])
def test_pressure_step_matches_oracle_chain(gpu_lib, oracle, gname, qprecond):
    g = dict(grid_cases())[gname]()
    st = gg.make_step_fields(g, seed=43)
    pr = q_props(qprecond)
    src, D = oracle.compute_qsource(st, pr)
    qc_ref, n_ref = oracle.cgsolveq(QProblem(grid=g, D=D, src=src, q=st.qc, c=st.c), pr)
    u_ref, w_ref, q_ref = oracle.corrector(st, qc_ref, D, pr)
    ctx = Context(g)
    ctx.step_grid(st)
    qc, u, w, q, stats = ctx.pressure_step(st, pr)
    ctx.close()
    assert stats.status == OK
    m = g.active_mask()
    assert np.linalg.norm(qc[m] - qc_ref[m]) <= 1e-9 * np.linalg.norm(qc_ref[m])
    for a, b, a0 in ((u, u_ref, st.u), (w, w_ref, st.w), (q, q_ref, st.q)):
        scale = max(np.abs(b - a0).max(), 1e-300)
        assert np.abs(a - b).max() <= 1e-8 * scale


@pytest.mark.parametrize("name", fixture_names())
def test_vertical_grid_functions_match_golden_bitwise(gpu_lib, name):
    """UpdateDZ (option 0) and SetFluxHeight on the device: the reference's bits."""
    g, qp, hp, props, d = load(name)
    st = step_fields(g, d)
    vf = vgrid_fields(g, d)
    ctx = Context(g)
    ctx.step_grid(st)
    for k, val in zip(("udz_ctop", "udz_etop", "udz_dzz", "udz_ctopold", "udz_etopold", "udz_dzzold"),
                      ctx.update_dz(vf)):
        assert np.array_equal(val, d[k]), k
    for sb in (0.0, 0.3):
        vf.smoothbot = sb
        dzf, dzz = ctx.set_flux_height(vf)
        tag = "sfh%d" % int(round(10 * sb))
        assert np.array_equal(dzf, d[tag + "_dzf"]) and np.array_equal(dzz, d[tag + "_dzz"])
    ctx.close()


@pytest.mark.parametrize("gname", [n for n, _ in grid_cases()])
def test_vertical_grid_functions_match_oracle_bitwise(gpu_lib, oracle, gname):
    g = dict(grid_cases())[gname]()
    st = gg.make_step_fields(g, seed=45)
    ctx = Context(g)
    ctx.step_grid(st)
    for sb in (0.0, 0.25):
        vf = gg.make_vgrid_fields(g, seed=46, smoothbot=sb)
        for a, b in zip(ctx.update_dz(vf), oracle.update_dz(vf)):
            assert np.array_equal(a, b)
        for a, b in zip(ctx.set_flux_height(vf), oracle.set_flux_height(vf)):
            assert np.array_equal(a, b)
    ctx.close()
