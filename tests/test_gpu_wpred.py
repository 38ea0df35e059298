"""WPredictor (main/phys.c:2025-2287) on the device, through the C ABI: the
Adams-Bashforth start, the pressure gradient, first-order upwind advection,
horizontal diffusion and wall drag gathered per column in the reference's edge
order, and the vertical diffusion solve give the reference's bits (the oracle
is pinned bit for bit against the reference's WPredictor and its golden
vectors).

The nonhydrostatic step (WPredictor -> ComputeQSource -> CGSolveQ ->
Corrector in one call, main/phys.c:1271-1289) matches the oracle's chain of
the four functions: w and the histories after WPredictor bit for bit (they
leave the device only at the end), the correction within relative L2 1e-9
(the solve's parity bound), u, w, q within 1e-8 of the size of the
correction they received."""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.capi import Context, SolverError
from suntans_gb300.capi import OK
from suntans_gb300.grid import QProblem
from tests._cases import h_props, q_props
from tests._golden import fixture_names, load, props_for, wpred_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle():
    return Oracle("port")


def _grids():
    return {
        "tri_open": lambda: gg.delaunay_seamount(3000, 8000, 4000, Nkmax=20, sigma=1200, ctop_frac=0.2,
                                                 h_sigma=0.05, open_x0=True, seed=71),
        "quad": lambda: gg.quad_channel(24, 10, Nkmax=12, h_sigma=0.05, ctop_frac=0.3, seed=72),
        "tri_deep": lambda: gg.delaunay_seamount(1500, 4000, 2000, Nkmax=70, rstretch=1.01, sigma=600, seed=73),
    }


CASES = [("tri_open", dict()), ("tri_open", dict(nonlinear=0)), ("tri_open", dict(n=1)),
         ("quad", dict(n=2)), ("quad", dict(AB=2, CdW=0.0)), ("tri_deep", dict())]


@pytest.mark.parametrize("gname,kw", CASES)
def test_wpredictor_matches_oracle_bitwise(gpu_lib, oracle, gname, kw):
    g = _grids()[gname]()
    wf = gg.make_wpred_fields(g, seed=74, **kw)
    pr = h_props(1, dt=10.0)
    ctx = Context(g)
    ctx.step_grid(wf)
    w, cw, cw2 = ctx.wpredictor(wf, pr)
    ctx.close()
    w_o, cw_o, cw2_o = oracle.wpredictor(wf, pr)
    assert np.array_equal(w, w_o) and np.array_equal(cw, cw_o) and np.array_equal(cw2, cw2_o)
    assert np.any(w != wf.w)


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("tag", ["wp1_", "wp0_"])
def test_wpredictor_matches_golden(gpu_lib, name, tag):
    g, qp, hp, props, d = load(name)
    wf = wpred_fields(g, d, tag)
    ctx = Context(g)
    ctx.step_grid(wf)
    w, cw, cw2 = ctx.wpredictor(wf, props_for(props))
    ctx.close()
    assert np.array_equal(w, d[tag + "out_w"]) and np.array_equal(cw, d[tag + "out_Cn_W"])
    assert np.array_equal(cw2, d[tag + "out_Cn_W2"])


def test_unsupported_settings_are_refused(gpu_lib):
    g = _grids()["quad"]()
    ctx = Context(g)
    for kw in (dict(nonlinear=2), dict(conserveMomentum=1)):
        wf = gg.make_wpred_fields(g, seed=75, **kw)
        ctx.step_grid(wf)
        with pytest.raises(SolverError):
            ctx.wpredictor(wf, h_props(1))
    ctx.close()


@pytest.mark.parametrize("qprecond", [0, 1])
@pytest.mark.parametrize("gname,kw", [("tri_open", dict()), ("quad", dict(nonlinear=0, n=1))])
def test_nonhydrostatic_step_matches_oracle_chain(gpu_lib, oracle, gname, kw, qprecond):
    g = _grids()[gname]()
    st = gg.make_step_fields(g, seed=79)
    wf = dataclasses.replace(gg.make_wpred_fields(g, seed=76, **kw), w=st.w, q=st.q, utmp2=st.utmp2)
    pr = q_props(qprecond)
    w_o, cw_o, cw2_o = oracle.wpredictor(wf, pr)
    st_o = dataclasses.replace(st, w=w_o)
    src, D = oracle.compute_qsource(st_o, pr)
    qc_ref, _ = oracle.cgsolveq(QProblem(grid=g, D=D, src=src, q=st.qc, c=st.c), pr)
    u_ref, w_ref, q_ref = oracle.corrector(st_o, qc_ref, D, pr)
    ctx = Context(g)
    ctx.step_grid(st)
    qc, u, w, q, cw, cw2, stats = ctx.nonhydrostatic_step(st, wf, pr)
    ctx.close()
    assert stats.status == OK
    assert np.array_equal(cw, cw_o) and np.array_equal(cw2, cw2_o)
    m = g.active_mask()
    assert np.linalg.norm(qc[m] - qc_ref[m]) <= 1e-9 * np.linalg.norm(qc_ref[m])
    for a, b, a0 in ((u, u_ref, st.u), (w, w_ref, w_o), (q, q_ref, st.q)):
        scale = max(np.abs(b - a0).max(), 1e-300)
        assert np.abs(a - b).max() <= 1e-8 * scale


def test_nonhydrostatic_step_refuses_unsupported_settings(gpu_lib):
    g = _grids()["quad"]()
    st = gg.make_step_fields(g, seed=80)
    ctx = Context(g)
    ctx.step_grid(st)
    for kw in (dict(nonlinear=2), dict(conserveMomentum=1)):
        wf = gg.make_wpred_fields(g, seed=81, **kw)
        with pytest.raises(SolverError):
            ctx.nonhydrostatic_step(st, wf, q_props(1))
    ctx.close()
