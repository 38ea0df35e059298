"""The C restatement of the reference algorithm (oracle/cg_oracle.c) is pinned
bit-for-bit against the reference's own outputs: the golden vectors made by
tests/golden/make_golden.py from the reference's compiled main/phys.c, and --
where the reference tree is present -- the reference library itself on larger
seeded grids."""
import os

import numpy as np
import pytest

from oracle import oracle as om
from oracle.oracle import Oracle
from suntans_gb300 import gridgen as gg
from tests._cases import grid_cases, h_props, q_props
from tests._golden import example_names, fixture_names, load, load_example, props_for


@pytest.fixture(scope="module")
def port():
    om.build_port()
    return Oracle("port")


def test_fixtures_present():
    assert len(fixture_names()) >= 3


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("qprecond", [0, 1, 2])
def test_port_cgsolveq_matches_golden_bitwise(port, name, qprecond):
    g, qp, hp, props, d = load(name)
    q, n = port.cgsolveq(qp, props_for(props, qprecond=qprecond))
    assert n == int(d[f"n_qp{qprecond}"])
    assert np.array_equal(q, d[f"q_qp{qprecond}"])


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("hprecond", [0, 1])
def test_port_cgsolve_matches_golden_bitwise(port, name, hprecond):
    g, qp, hp, props, d = load(name)
    h, n = port.cgsolve(hp, props_for(props, hprecond=hprecond))
    assert n == int(d[f"n_hp{hprecond}"])
    assert np.array_equal(h, d[f"h_hp{hprecond}"])


@pytest.mark.parametrize("name", fixture_names())
def test_port_operators_match_golden_bitwise(port, name):
    g, qp, hp, props, d = load(name)
    x = d["x"]
    c = port.condition_q(g, qp.D, np.ones(g.n3))
    assert np.array_equal(c, d["condq"])
    coef0, _ = port.qcoefficients(g, qp.D, c, 0)
    coef1, fcoef1 = port.qcoefficients(g, qp.D, c, 1)
    assert np.array_equal(coef0, d["coef0"])
    assert np.array_equal(coef1, d["coef1"]) and np.array_equal(fcoef1, d["fcoef1"])
    assert np.array_equal(port.operator_q(g, qp.D, coef0, x), d["opq"])
    assert np.array_equal(port.operator_qc(g, coef1, fcoef1, x), d["opqc"])
    assert np.array_equal(port.preconditioner(g, coef0, x), d["precond"])
    hcoef, hfcoef = port.hcoefficients(g, hp.D, props_for(props))
    assert np.array_equal(hcoef, d["hcoef"]) and np.array_equal(hfcoef, d["hfcoef"])
    assert np.array_equal(port.operator_h(g, hcoef, hfcoef, x[:g.Nc]), d["oph"])


def test_golden_cover_edge_cases():
    """The fixtures hold the cases the solvers special-case: dry top layers
    (ctop > 0), single-level wet columns (ctop = Nk-1), type-3 boundary cells,
    walls, quads and triangles."""
    seen = dict(ctop=False, single=False, bdy=False, quad=False, tri=False)
    for name in fixture_names():
        g, *_ = load(name)
        seen["ctop"] |= bool((g.ctop > 0).any())
        seen["single"] |= bool((g.ctop == g.Nk - 1).any())
        seen["bdy"] |= bool(g.celldist[2] > g.celldist[1])
        seen["quad"] |= g.maxfaces == 4
        seen["tri"] |= g.maxfaces == 3
    assert all(seen.values()), seen


ref_present = om.build_ref() is not None if not om.available("ref") else True


@pytest.mark.skipif(not ref_present, reason="reference sources not present on this host")
@pytest.mark.parametrize("gname", [n for n, _ in grid_cases()[:2]] + ["tri400_shallow"])
def test_port_matches_reference_library(port, gname):
    ref = Oracle("ref")
    g = dict(grid_cases())[gname]()
    qp = gg.make_q_problem(g, seed=8, q0_sigma=0.02)
    for qpc in (0, 1, 2):
        a, na = port.cgsolveq(qp, q_props(qpc))
        b, nb = ref.cgsolveq(qp, q_props(qpc))
        assert na == nb and np.array_equal(a, b)
    hp = gg.make_h_problem(g, seed=9)
    for hpc in (0, 1):
        a, na = port.cgsolve(hp, h_props(hpc))
        b, nb = ref.cgsolve(hp, h_props(hpc))
        assert na == nb and np.array_equal(a, b)
    st = gg.make_step_fields(g, seed=10)
    pr = q_props(1)
    sa, Da = port.compute_qsource(st, pr)
    sb, Db = ref.compute_qsource(st, pr)
    assert np.array_equal(sa, sb) and np.array_equal(Da, Db)
    qc = port.cgsolveq(gg.QProblem(grid=g, D=Da, src=sa, q=st.qc, c=st.c), pr)[0]
    for x, y in zip(port.corrector(st, qc, Da, pr), ref.corrector(st, qc, Da, pr)):
        assert np.array_equal(x, y)
    if g.dz is not None:
        vf = gg.make_vgrid_fields(g, seed=11, smoothbot=0.2)
        for x, y in zip(port.update_dz(vf), ref.update_dz(vf)):
            assert np.array_equal(x, y)
        for x, y in zip(port.set_flux_height(vf), ref.set_flux_height(vf)):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("name", fixture_names())
def test_port_step_functions_match_golden_bitwise(port, name):
    """ComputeQSource and Corrector of the restatement reproduce the reference's bits."""
    from tests._golden import step_fields
    g, qp, hp, props, d = load(name)
    st = step_fields(g, d)
    src, D = port.compute_qsource(st, props_for(props))
    assert np.array_equal(src, d["qs_src"]) and np.array_equal(D, d["qs_D"])
    u, w, q = port.corrector(st, d["q_qp1"], d["qs_D"], props_for(props))
    assert np.array_equal(u, d["corr_u"]) and np.array_equal(w, d["corr_w"]) and np.array_equal(q, d["corr_q"])
    # the fixtures exercise both branches of the edge and column conditions
    assert np.any(u != d["u"]) and np.any(w != d["w"]) and np.any(q != d["qtot"])


@pytest.mark.parametrize("name", fixture_names())
def test_port_vertical_grid_functions_match_golden_bitwise(port, name):
    """UpdateDZ (option 0) and SetFluxHeight of the restatement reproduce the reference's bits."""
    from tests._golden import vgrid_fields
    g, qp, hp, props, d = load(name)
    vf = vgrid_fields(g, d)
    for k, val in zip(("udz_ctop", "udz_etop", "udz_dzz", "udz_ctopold", "udz_etopold", "udz_dzzold"),
                      port.update_dz(vf)):
        assert np.array_equal(val, d[k]), k
    assert np.any(d["udz_ctop"] != d["vg_ctop"])  # the free surface moved some tops
    for sb in (0.0, 0.3):
        vf.smoothbot = sb
        dzf, dzz = port.set_flux_height(vf)
        tag = "sfh%d" % int(round(10 * sb))
        assert np.array_equal(dzf, d[tag + "_dzf"]) and np.array_equal(dzz, d[tag + "_dzz"])


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("nl", [0, 1])
def test_port_upredictor_matches_golden_bitwise(port, name, nl):
    """The whole of UPredictor (vertical solve, free-surface right-hand side,
    CGSolve, velocity update, UpdateDZ, boundary fluxes) reproduces the
    reference's bits, and its pieces compose to it."""
    from tests._golden import upred_fields, vgrid_fields
    g, qp, hp, props, d = load(name)
    vf = vgrid_fields(g, d)
    uf = upred_fields(g, d, nl)
    pr = props_for(props)
    r = port.upredictor(uf, vf, pr)
    pre = f"up{nl}_out_"
    for k in ("u", "h", "utmp", "E", "D", "ctop", "etop", "dzz", "active"):
        assert np.array_equal(r[k], d[pre + k]), k
    assert r["niters"] == int(d[pre + "niters"]) and r["nnan"] == 0
    ut, E, D, nnan = port.upredictor_vertical(uf, pr)
    ce = uf.edgep
    eo = g.eoff
    rows = np.concatenate([np.arange(eo[j], eo[j + 1]) for j in ce])
    assert np.array_equal(D, r["D"]) and np.array_equal(E[rows], r["E"][rows])
    assert np.array_equal(ut[rows], r["utmp"][rows])
    assert np.any(r["ctop"] != g.ctop) or np.any(r["etop"] != uf.etop)


@pytest.mark.parametrize("case", ["drag", "noslip_all", "no_lax", "no_advection"])
def test_port_upredictor_matches_reference_library(port, case):
    if not om.available("ref"):
        pytest.skip("reference library not built here")
    ref = Oracle("ref")
    g = gg.delaunay_seamount(400, 3000, 1500, Nkmax=10, sigma=400, ctop_frac=0.3, h_sigma=0.05, open_x0=True,
                             seed=41)
    kw = dict(nonlinear=1, thetaM=0.5, laxWendroff_Vertical=1.0, noslip_frac=0.2)
    if case == "no_lax":
        kw["laxWendroff_Vertical"] = 0.0
    if case == "no_advection":
        kw["thetaM"] = -1.0
    uf = gg.make_upred_fields(g, seed=42, **kw)
    if case == "noslip_all":      # includes single-layer edges (the stale scratch read of phys.c:2864)
        uf.CdB[:] = -1.0
        uf.CdT[:] = -1.0
    vf = gg.make_vgrid_fields(g, seed=43)
    pr = h_props(1, dt=10.0)
    a, b = port.upredictor(uf, vf, pr), ref.upredictor(uf, vf, pr)
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.parametrize("name", fixture_names())
@pytest.mark.parametrize("tag", ["wp1_", "wp0_"])
def test_port_wpredictor_matches_golden_bitwise(port, name, tag):
    """WPredictor (Adams-Bashforth, pressure gradient, upwind advection,
    horizontal diffusion and wall drag, the vertical diffusion solve)
    reproduces the reference's bits."""
    from tests._golden import wpred_fields
    g, qp, hp, props, d = load(name)
    wf = wpred_fields(g, d, tag)
    w, cw, cw2 = port.wpredictor(wf, props_for(props))
    assert np.array_equal(w, d[tag + "out_w"]) and np.array_equal(cw, d[tag + "out_Cn_W"])
    assert np.array_equal(cw2, d[tag + "out_Cn_W2"])
    assert np.any(w != wf.w)


@pytest.mark.parametrize("kw", [dict(), dict(nonlinear=0), dict(n=1), dict(n=2), dict(AB=2),
                                dict(conserveMomentum=1), dict(CdW=0.0, nu_H=0.0)])
def test_port_wpredictor_matches_reference_library(port, kw):
    if not om.available("ref"):
        pytest.skip("reference library not built here")
    ref = Oracle("ref")
    g = gg.delaunay_seamount(400, 3000, 1500, Nkmax=10, sigma=400, ctop_frac=0.3, h_sigma=0.05, open_x0=True,
                             seed=44)
    wf = gg.make_wpred_fields(g, seed=45, **kw)
    pr = h_props(1, dt=10.0)
    for a, b in zip(port.wpredictor(wf, pr), ref.wpredictor(wf, pr)):
        assert np.array_equal(a, b)


# the reference's own example triangulations (main/gridio.c input files), as solver grids
_EXAMPLES = om.ref_examples_dir() or ""
_EXAMPLE_GRIDS = [("riverplume/grids/hex", 7), ("riverplume/grids/hybrid", 7), ("riverplume/grids/quad", 4),
                  ("riverplume/grids/tri", 3), ("heatflux/rundata", 4)]


def _example_grid(folder, mf, seed, **kw):
    from suntans_gb300 import formats as fm
    d = os.path.join(_EXAMPLES, folder)
    if not os.path.isfile(os.path.join(d, "cells.dat")):
        pytest.skip("the reference's example grids are not present on this host")
    mg = fm.read_main_grid(d, maxfaces=mf)
    g = gg.from_main_grid(mg, Nkmax=8, ctop_frac=0.2, h_sigma=0.1, seed=seed, name=folder, **kw)
    assert g.Ne == mg.Ne  # the edges rebuilt from the cells are the file's edges
    return g


@pytest.mark.skipif(not ref_present, reason="reference sources not present on this host")
@pytest.mark.parametrize("folder,mf", _EXAMPLE_GRIDS, ids=[f for f, _ in _EXAMPLE_GRIDS])
def test_port_matches_reference_library_on_example_grids(port, folder, mf):
    """CGSolveQ (qprecond 0, 1, 2) and CGSolve (hprecond 0, 1) bit for bit on
    the reference's example grids: hexagons and mixed cells up to 7 faces,
    quads, triangles; partial top cells and a perturbed free surface."""
    g = _example_grid(folder, mf, seed=12)
    ref = Oracle("ref")
    qp = gg.make_q_problem(g, seed=13, q0_sigma=0.02)
    for qpc in (0, 1, 2):
        a, na = port.cgsolveq(qp, q_props(qpc))
        b, nb = ref.cgsolveq(qp, q_props(qpc))
        assert na == nb and na > 2 and np.array_equal(a, b)
    hp = gg.make_h_problem(g, seed=14)
    for hpc in (0, 1):
        a, na = port.cgsolve(hp, h_props(hpc))
        b, nb = ref.cgsolve(hp, h_props(hpc))
        assert na == nb and na > 2 and np.array_equal(a, b)


@pytest.mark.parametrize("name", example_names())
def test_port_matches_example_golden_bitwise(port, name):
    """The oracle's solvers on the stored example-grid cases: the reference's
    solutions and iteration counts, bit for bit."""
    g, qp, hp, props, d = load_example(name)
    assert int(g.nfaces.max()) >= 4
    for qpc in (0, 1, 2):
        q, n = port.cgsolveq(qp, props_for(props, qprecond=qpc))
        assert n == int(d[f"n_qp{qpc}"]) and np.array_equal(q, d[f"q_qp{qpc}"])
    for hpc in (0, 1):
        h, n = port.cgsolve(hp, props_for(props, hprecond=hpc))
        assert n == int(d[f"n_hp{hpc}"]) and np.array_equal(h, d[f"h_hp{hpc}"])


@pytest.mark.skipif(not ref_present, reason="reference sources not present on this host")
@pytest.mark.parametrize("folder,mf", _EXAMPLE_GRIDS[:2], ids=[f for f, _ in _EXAMPLE_GRIDS[:2]])
def test_port_steps_match_reference_library_on_example_grids(port, folder, mf):
    """The steps around the solves on hexagon / maxFaces-7 grids, bit for bit:
    ComputeQSource, Corrector, UpdateDZ, SetFluxHeight, WPredictor (with and
    without advection) and the whole UPredictor (cells of up to 7 faces in
    the edge loops, the per-cell face sums and the free-surface solve)."""
    g = _example_grid(folder, mf, seed=15, scale=0.02)
    ref = Oracle("ref")
    st = gg.make_step_fields(g, seed=16)
    pr = q_props(1)
    sa, Da = port.compute_qsource(st, pr)
    sb, Db = ref.compute_qsource(st, pr)
    assert np.array_equal(sa, sb) and np.array_equal(Da, Db)
    qc = port.cgsolveq(gg.QProblem(grid=g, D=Da, src=sa, q=st.qc, c=st.c), pr)[0]
    for x, y in zip(port.corrector(st, qc, Da, pr), ref.corrector(st, qc, Da, pr)):
        assert np.array_equal(x, y)
    vf = gg.make_vgrid_fields(g, seed=17, smoothbot=0.2)
    for x, y in zip(port.update_dz(vf), ref.update_dz(vf)):
        assert np.array_equal(x, y)
    for x, y in zip(port.set_flux_height(vf), ref.set_flux_height(vf)):
        assert np.array_equal(x, y)
    hp = h_props(1, dt=10.0)
    for kw in (dict(), dict(nonlinear=0, n=1)):
        wf = gg.make_wpred_fields(g, seed=18, **kw)
        for x, y in zip(port.wpredictor(wf, hp), ref.wpredictor(wf, hp)):
            assert np.array_equal(x, y)
    uf = gg.make_upred_fields(g, seed=19)
    vf = gg.make_vgrid_fields(g, seed=20)
    a, b = port.upredictor(uf, vf, hp), ref.upredictor(uf, vf, hp)
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_summation_order_moves_iterations_not_solution(port):
    """On the reference's riverplume hybrid grid with qprecond 2 (a poorly
    conditioned block-Jacobi solve, 394 iterations) the port with its inner
    products added pairwise instead of sequentially stops at a different
    iteration (375), while its solution stays within round-off of the
    reference's.  This is why the device tests compare iteration counts
    against the span of the two orders rather than one count."""
    from tests._cases import rel_l2
    g, qp, hp, props, d = load_example("riverplume_hybrid")
    pr = props_for(props, qprecond=2)
    n_seq, n_pair = port.iteration_span(qp, pr)
    assert n_seq == int(d["n_qp2"])
    assert abs(n_pair - n_seq) > max(4, int(0.03 * n_seq))
    port.lib.sgo_set_sum_order(1)
    try:
        q, n = port.cgsolveq(qp, pr)
    finally:
        port.lib.sgo_set_sum_order(0)
    assert n == n_pair
    assert rel_l2(q, d["q_qp2"], g.active_mask()) <= 1e-9


def test_port_matches_lockexchange_run_bitwise(port):
    """The lock-exchange channel fixture records the reference model's own
    solves over a 10-step nonhydrostatic run (make_lockexchange_golden.py):
    the port, given each solve's recorded inputs, returns the reference's
    solution bit for bit with its iteration count."""
    from tests._golden import load_lockexchange
    d, props, grid_at, q_problem, h_problem = load_lockexchange()
    assert list(d["q_steps"]) == [1, 5, 10] and list(d["h_steps"]) == list(range(1, 11))
    for s in d["q_steps"]:
        p, ref, n = q_problem(int(s))
        q, nq = port.cgsolveq(p, props)
        assert nq == n and np.array_equal(q, ref)
    for s in d["h_steps"]:
        p, ref, n = h_problem(int(s))
        h, nh = port.cgsolve(p, props)
        assert nh == n and np.array_equal(h, ref)
