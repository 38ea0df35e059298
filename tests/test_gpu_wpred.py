"""WPredictor (main/phys.c:2025-2287) on the device, through the C ABI: the
Adams-Bashforth start, the pressure gradient, first-order upwind advection,
horizontal diffusion and wall drag gathered per column in the reference's edge
order, and the vertical diffusion solve give the reference's bits (the oracle
is pinned bit for bit against the reference's WPredictor and its golden
vectors)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.capi import Context, SolverError
from tests._cases import h_props
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
