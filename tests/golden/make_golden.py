"""Generates the golden vectors in tests/golden/*.npz from the REFERENCE itself.

Run where the SUNTANS reference sources are present (they are compiled into
oracle/_ref/libsuntans_ref.so by `make -C oracle ref`, the reference's own
main/phys.c wrapped by oracle/ref_harness.c):

    python tests/golden/make_golden.py

Each fixture stores a small seeded grid with every input array the solvers
read, and the reference's outputs for:
  CGSolveQ with qprecond 0, 1, 2 (solution q and the iteration count),
  CGSolve with hprecond 0, 1 (solution h and the iteration count),
  QCoefficients (qprecond 0 and 1), OperatorQ, OperatorQC, ConditionQ,
  Preconditioner, HCoefficients and OperatorH on a seeded vector,
  ComputeQSource on seeded velocity fields and Corrector with the qprecond-1
  solution as the pressure correction (the steps around CGSolveQ),
  UpdateDZ (option 0) and SetFluxHeight (smoothbot 0 and 0.3) on a seeded
  free surface and edge velocity,
  UPredictor with CGSolve (main/phys.c:2579-3077) on seeded drag, viscosity
  and velocity fields, with and without implicit vertical advection,
  WPredictor (main/phys.c:2025-2287) with first-order upwind advection (AB3)
  and without advection on the first step.
The inputs are stored (not regenerated) so that the check is bit-exact on any
host: tests/test_oracle.py runs the C restatement (oracle/cg_oracle.c) on them
and requires identical bits.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as om  # noqa: E402
from suntans_gb300 import gridgen as gg  # noqa: E402
from suntans_gb300.grid import SolverProps  # noqa: E402

GRID_FIELDS = ("nfaces", "neigh", "face", "Nk", "Nke", "ctop", "cellp", "celldist", "Ac", "df", "dg", "dzz", "dzf")


def cases():
    return {
        "quad8x6": gg.quad_channel(8, 6, Nkmax=8, h_sigma=0.05, ctop_frac=0.3, seed=21),
        "tri120_open": gg.delaunay_seamount(120, 1000, 500, Nkmax=8, sigma=150, ctop_frac=0.2, h_sigma=0.05,
                                            open_x0=True, seed=22),
        "tri80_shallow": gg.delaunay_seamount(80, 600, 300, Nkmax=4, H0=4.0, amp=3.6, sigma=100, ctop_frac=0.5,
                                              h_sigma=0.05, seed=23),
    }


def main():
    if om.build_ref() is None:
        raise SystemExit("reference sources not found; cannot generate golden vectors")
    ref = om.Oracle("ref")
    for name, g in cases().items():
        g.validate()
        out = {f: getattr(g, f) for f in GRID_FIELDS}
        out["sizes"] = np.array([g.Nc, g.Ne, g.maxfaces, g.Nkmax], dtype=np.int32)
        qp = gg.make_q_problem(g, seed=31, q0_sigma=0.01)
        hp = gg.make_h_problem(g, seed=32)
        out.update(qD=qp.D, src=qp.src, q0=qp.q, c0=qp.c, hD=hp.D, htmp=hp.htmp, h0=hp.h)
        props = dict(qmaxiters=3000, qepsilon=1e-10, resnorm=1.0, dt=10.0, theta=0.55, grav=9.81,
                     maxiters=3000, epsilon=1e-10)
        out["props"] = np.array([props["qmaxiters"], props["qepsilon"], props["resnorm"], props["dt"],
                                 props["theta"], props["grav"], props["maxiters"], props["epsilon"]])
        for qpc in (0, 1, 2):
            q, n = ref.cgsolveq(qp, SolverProps(qprecond=qpc, **props))
            out[f"q_qp{qpc}"] = q
            out[f"n_qp{qpc}"] = np.array(n)
        for hpc in (0, 1):
            h, n = ref.cgsolve(hp, SolverProps(hprecond=hpc, **props))
            out[f"h_hp{hpc}"] = h
            out[f"n_hp{hpc}"] = np.array(n)
        rng = np.random.default_rng(33)
        x = rng.normal(size=g.n3)
        out["x"] = x
        c = ref.condition_q(g, qp.D, np.ones(g.n3))
        out["condq"] = c
        coef0, _ = ref.qcoefficients(g, qp.D, c, 0)
        coef1, fcoef1 = ref.qcoefficients(g, qp.D, c, 1)
        out.update(coef0=coef0, coef1=coef1, fcoef1=fcoef1)
        out["opq"] = ref.operator_q(g, qp.D, coef0, x)
        out["opqc"] = ref.operator_qc(g, coef1, fcoef1, x)
        out["precond"] = ref.preconditioner(g, coef0, x)
        hcoef, hfcoef = ref.hcoefficients(g, hp.D, SolverProps(**props))
        out.update(hcoef=hcoef, hfcoef=hfcoef)
        out["oph"] = ref.operator_h(g, hcoef, hfcoef, x[:g.Nc])
        st = gg.make_step_fields(g, seed=34)
        out.update(normal=g.normal, grad=g.grad, u=st.u, utmp2=st.utmp2, w=st.w, wtmp2=st.wtmp2, qtot=st.q,
                   etop=st.etop, edgep=st.edgep, edgedist=st.edgedist)
        qs_src, qs_D = ref.compute_qsource(st, SolverProps(**props))
        out.update(qs_src=qs_src, qs_D=qs_D)
        cu, cw, cq = ref.corrector(st, out["q_qp1"], qs_D, SolverProps(**props))
        out.update(corr_u=cu, corr_w=cw, corr_q=cq)
        vf = gg.make_vgrid_fields(g, seed=35)
        out.update(vg_dz=g.dz, vg_dv=g.dv, vg_h=vf.h, vg_u=vf.u, vg_dzbot=vf.dzbot, vg_Nkc=vf.Nkc,
                   vg_ctop=vf.ctop, vg_etop=vf.etop, vg_dzz=vf.dzz)
        for k, val in zip(("udz_ctop", "udz_etop", "udz_dzz", "udz_ctopold", "udz_etopold", "udz_dzzold"),
                          ref.update_dz(vf)):
            out[k] = val
        for sb in (0.0, 0.3):
            vf.smoothbot = sb
            dzf, dzz2 = ref.set_flux_height(vf)
            tag = "sfh%d" % int(round(10 * sb))
            out[tag + "_dzf"] = dzf
            out[tag + "_dzz"] = dzz2
        for nl in (0, 1):
            uf = gg.make_upred_fields(g, seed=36 + nl, nonlinear=nl)
            pre = f"up{nl}_"
            for k in ("u", "w", "h", "utmp", "tau_T", "CdT", "CdB", "nu_tv", "nu_lax", "etop", "edgep", "edgedist",
                      "bedgep", "bedgedist", "mark", "n1", "n2"):
                out[pre + k] = getattr(uf, k)
            out[pre + "par"] = np.array([uf.nu, uf.laxWendroff_Vertical, uf.thetaM, uf.nonlinear])
            r = ref.upredictor(uf, vf, SolverProps(**props))
            for k in ("u", "h", "utmp", "E", "D", "ctop", "etop", "dzz", "active"):
                out[pre + "out_" + k] = r[k]
            out[pre + "out_niters"] = np.array(r["niters"])
        for tag, kw in (("wp1_", dict(nonlinear=1, n=5, AB=3)), ("wp0_", dict(nonlinear=0, n=1, AB=3))):
            wf = gg.make_wpred_fields(g, seed=38, **kw)
            for k in ("w", "Cn_W", "Cn_W2", "q", "nu_tv", "nu_lax", "utmp2"):
                out[tag + k] = getattr(wf, k)
            out[tag + "par"] = np.array([wf.nu, wf.nu_H, wf.CdW, wf.laxWendroff_Vertical, wf.nonlinear,
                                         wf.conserveMomentum, wf.n, wf.AB])
            w, cw, cw2 = ref.wpredictor(wf, SolverProps(**props))
            out.update({tag + "out_w": w, tag + "out_Cn_W": cw, tag + "out_Cn_W2": cw2})
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: Nc={g.Nc} n3={g.n3} iters q={[int(out[f'n_qp{k}']) for k in range(3)]} "
              f"h={[int(out[f'n_hp{k}']) for k in range(2)]} {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
