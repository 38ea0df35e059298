"""UPredictor (main/phys.c:2579-3077) on the device, through the C ABI.

* The vertical predictor (U***, E, D), the free-surface right-hand side and
  the post-solve steps (dry clip, velocity update, UpdateDZ, type-2 / type-3
  boundaries) are plain FP64 arithmetic in the reference's order without
  contraction: their device results equal the oracle's bit for bit (the oracle
  is pinned bit for bit against the reference's whole UPredictor and its
  golden vectors).
* The whole predictor with CGSolve between keeps everything in HBM; it matches
  the oracle's whole UPredictor with U***, E and D bit for bit, the new free
  surface within relative L2 1e-9 (the solve's parity bound) and u within
  1e-8 of the size of the free-surface term it received.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from suntans_gb300.capi import BREAKDOWN, Context, OK, SolverError
from tests._cases import h_props
from tests._golden import fixture_names, load, props_for, upred_fields, vgrid_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle():
    return Oracle("port")


def _grids():
    return {
        "tri_open": lambda: gg.delaunay_seamount(3000, 8000, 4000, Nkmax=20, sigma=1200, ctop_frac=0.2,
                                                 h_sigma=0.05, open_x0=True, seed=51),
        "quad_open": lambda: gg.quad_channel(24, 10, Nkmax=12, h_sigma=0.05, ctop_frac=0.3, open_x0=True, seed=52),
        "tri_deep": lambda: gg.delaunay_seamount(1500, 4000, 2000, Nkmax=70, rstretch=1.01, sigma=600, seed=53),
    }


CASES = [("tri_open", dict()), ("tri_open", dict(nonlinear=0)), ("quad_open", dict(thetaM=-1.0)),
         ("quad_open", dict(laxWendroff_Vertical=0.0, noslip_frac=0.5)), ("tri_deep", dict())]


def _ctx(g, uf):
    ctx = Context(g)
    ctx.step_grid(uf)
    ctx.upredictor_grid(uf)
    return ctx


def _oracle_chain(oracle, uf, vf, pr):
    """The oracle's UPredictor composed from its pieces, with the intermediate
    state the device pieces take."""
    g = uf.grid
    utmp, E, D, nnan = oracle.upredictor_vertical(uf, pr)
    h = np.array(uf.h, copy=True)
    h[g.cellp[g.celldist[1]:g.celldist[2]]] = 0.0
    vf1 = gg.make_vgrid_fields(g, seed=0)
    vf1.h, vf1.dzbot, vf1.Nkc, vf1.ctop, vf1.etop, vf1.dzz = h, vf.dzbot, vf.Nkc, g.ctop, uf.etop, g.dzz
    ctop1, etop1, dzz1 = oracle.update_dz(vf1)[:3]
    ut = utmp.copy()
    eo = g.eoff
    for t in range(uf.bedgedist[2], uf.bedgedist[5]):
        j = uf.bedgep[t]
        ut[eo[j] + etop1[j]:eo[j + 1]] = 0.0 * uf.n1[j] + 0.0 * uf.n2[j]
    g1 = _with_state(g, ctop1, dzz1)
    htmp = oracle.upredictor_rhs(uf, pr, ut, h=h, grid=g1, etop=etop1)
    return dict(utmp=ut, E=E, D=D, h1=h, ctop1=ctop1, etop1=etop1, dzz1=dzz1, htmp=htmp, g1=g1)


def _with_state(g, ctop, dzz):
    import copy
    g1 = copy.copy(g)
    g1.ctop = np.ascontiguousarray(ctop, dtype=np.int32)
    g1.dzz = np.ascontiguousarray(dzz, dtype=np.float64)
    return g1


@pytest.mark.parametrize("gname,kw", CASES)
def test_vertical_and_rhs_match_oracle_bitwise(gpu_lib, oracle, gname, kw):
    g = _grids()[gname]()
    uf = gg.make_upred_fields(g, seed=61, **kw)
    pr = h_props(1, dt=20.0)
    ctx = _ctx(g, uf)
    ut, E, D = ctx.upredictor_vertical(uf, pr)
    ut_o, E_o, D_o, nnan = oracle.upredictor_vertical(uf, pr)
    assert nnan == 0
    assert np.array_equal(ut, ut_o) and np.array_equal(D, D_o)
    rows = np.concatenate([np.arange(g.eoff[j], g.eoff[j + 1]) for j in uf.edgep])
    assert np.array_equal(E[rows], E_o[rows])
    assert np.any(ut != uf.utmp) and np.all(D[uf.edgep] > 0)
    ht = ctx.upredictor_rhs(uf, pr, ut_o)
    ht_o = oracle.upredictor_rhs(uf, pr, ut_o)
    assert np.array_equal(ht, ht_o)
    ctx.close()


@pytest.mark.parametrize("gname,kw", CASES[:3])
def test_finish_matches_oracle_bitwise(gpu_lib, oracle, gname, kw):
    g = _grids()[gname]()
    uf = gg.make_upred_fields(g, seed=62, **kw)
    vf = gg.make_vgrid_fields(g, seed=63)
    pr = h_props(1, dt=20.0)
    s = _oracle_chain(oracle, uf, vf, pr)
    # a free surface after the solve, with some cells dry (clipped) and some type-3 values
    rng = np.random.default_rng(64)
    h = s["h1"] + rng.normal(0.0, 0.02, g.Nc)
    dry = rng.random(g.Nc) < 0.05
    h[dry] = -g.dv[dry] - 1.0
    h_o, act_o, u_o = oracle.upredictor_velocity(uf, vf, pr, s["utmp"], s["E"], h, grid=s["g1"], etop=s["etop1"])
    vf2 = gg.make_vgrid_fields(g, seed=0)
    vf2.h, vf2.dzbot, vf2.Nkc, vf2.ctop, vf2.etop, vf2.dzz = h_o, vf.dzbot, vf.Nkc, s["ctop1"], s["etop1"], s["dzz1"]
    ctop2, etop2, dzz2 = oracle.update_dz(vf2)[:3]
    u_o = oracle.upredictor_boundary(uf, s["utmp"], u_o, grid=_with_state(g, ctop2, dzz2), etop=etop2)
    ctx = _ctx(g, uf)
    h_d, act_d, u_d, ct_d, et_d, zz_d = ctx.upredictor_finish(uf, vf, pr, s["utmp"], s["E"], h, s["ctop1"],
                                                              s["etop1"], s["dzz1"])
    ctx.close()
    assert np.array_equal(h_d, h_o) and np.array_equal(act_d, act_o)
    assert np.array_equal(ct_d, ctop2) and np.array_equal(et_d, etop2) and np.array_equal(zz_d, dzz2)
    assert np.array_equal(u_d, u_o)
    assert np.any(act_o == 0) and np.any(act_o == 1)
    if g.celldist[2] > g.celldist[1]:
        m3 = np.nonzero(uf.mark == 3)[0]
        rows = np.concatenate([np.arange(g.eoff[j] + etop2[j], g.eoff[j + 1]) for j in m3])
        assert np.any(u_o[rows] != uf.u[rows])   # the continuity flux was written


@pytest.mark.parametrize("gname,kw", CASES)
def test_whole_upredictor_matches_oracle(gpu_lib, oracle, gname, kw):
    g = _grids()[gname]()
    uf = gg.make_upred_fields(g, seed=65, **kw)
    vf = gg.make_vgrid_fields(g, seed=66)
    pr = h_props(1, dt=20.0)
    o = oracle.upredictor(uf, vf, pr)
    ctx = _ctx(g, uf)
    d = ctx.upredictor(uf, vf, pr)
    ctx.close()
    assert d["stats"].status == OK
    for k in ("utmp", "D"):
        assert np.array_equal(d[k], o[k]), k
    rows = np.concatenate([np.arange(g.eoff[j], g.eoff[j + 1]) for j in uf.edgep])
    assert np.array_equal(d["E"][rows], o["E"][rows])
    comp = g.cellp[:g.celldist[1]]
    assert np.linalg.norm(d["h"][comp] - o["h"][comp]) <= 1e-9 * np.linalg.norm(o["h"][comp])
    assert abs(d["niters"] - o["niters"]) <= max(4, 0.03 * o["niters"])
    assert np.array_equal(d["ctop"], o["ctop"]) and np.array_equal(d["etop"], o["etop"])
    assert np.array_equal(d["active"], o["active"])
    assert np.abs(d["dzz"] - o["dzz"]).max() <= 1e-9 * max(np.abs(o["dzz"]).max(), 1.0)
    scale = max(np.abs(o["u"] - o["utmp"]).max(), 1e-300)
    assert np.abs(d["u"] - o["u"]).max() <= 1e-8 * scale


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("nl", [0, 1])
def test_upredictor_pieces_match_golden(gpu_lib, name, nl):
    """The vertical predictor reproduces the reference's golden U***, E and D
    (stored from the reference's whole UPredictor) on the computational edges."""
    g, qp, hp, props, d = load(name)
    vf = vgrid_fields(g, d)
    uf = upred_fields(g, d, nl)
    ctx = Context(g)
    ctx.step_grid(uf)
    ut, E, D = ctx.upredictor_vertical(uf, props_for(props))
    ctx.close()
    pre = f"up{nl}_out_"
    rows = np.concatenate([np.arange(g.eoff[j], g.eoff[j + 1]) for j in uf.edgep])
    assert np.array_equal(D, d[pre + "D"])
    assert np.array_equal(E[rows], d[pre + "E"][rows]) and np.array_equal(ut[rows], d[pre + "utmp"][rows])


def test_nan_in_predictor_is_reported(gpu_lib):
    g = _grids()["quad_open"]()
    uf = gg.make_upred_fields(g, seed=67)
    j = int(uf.edgep[3])
    uf.utmp[g.eoff[j] + uf.etop[j]] = np.nan
    ctx = _ctx(g, uf)
    with pytest.raises(SolverError) as ei:
        ctx.upredictor_vertical(uf, h_props(1))
    assert ei.value.args[0].endswith(f"(status {BREAKDOWN})") and "NaN" in ctx.error()
    # the context stays usable
    uf2 = gg.make_upred_fields(g, seed=67)
    ctx.upredictor_vertical(uf2, h_props(1))
    ctx.close()


def test_bad_etop_is_refused(gpu_lib):
    g = _grids()["quad_open"]()
    uf = gg.make_upred_fields(g, seed=68)
    et = uf.etop.copy()
    et[5] = g.Nke[5]
    ctx = _ctx(g, uf)
    with pytest.raises(SolverError):
        ctx.upredictor_vertical(uf, h_props(1), etop=et)
    ctx.close()
