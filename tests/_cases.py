"""Seeded grids and problems shared by the parity tests (small enough for the oracle)."""
from __future__ import annotations

import numpy as np

from suntans_gb300 import gridgen as gg
from suntans_gb300.grid import SolverProps


def grid_cases():
    """(name, builder) pairs; builders are cheap and deterministic."""
    return [
        ("quad16x8", lambda: gg.quad_channel(16, 8, Nkmax=12, h_sigma=0.05, ctop_frac=0.3, seed=2)),
        ("tri600_open", lambda: gg.delaunay_seamount(600, 2000, 1000, Nkmax=15, sigma=300, ctop_frac=0.2,
                                                    h_sigma=0.05, open_x0=True, seed=5)),
        ("quad64x16x32", lambda: gg.quad_channel(64, 16, Nkmax=32, h_sigma=0.01, seed=3)),
        ("tri3000_partial", lambda: gg.delaunay_seamount(3000, 4000, 2000, Nkmax=30, sigma=500,
                                                        rstretch=1.05, ctop_frac=0.05, h_sigma=0.02, seed=7)),
        ("tri400_shallow", lambda: gg.delaunay_seamount(400, 1000, 500, Nkmax=6, H0=6.0, amp=5.5, sigma=150,
                                                       ctop_frac=0.5, h_sigma=0.05, seed=11)),
        ("hybrid30x12", lambda: gg.hybrid_channel(30, 12, Nkmax=10, h_sigma=0.05, ctop_frac=0.2, seed=13,
                                                  open_x0=True)),
    ]


def active_mask(g):
    return g.active_mask()


def rel_l2(a, b, mask=None):
    if mask is not None:
        a, b = a[mask], b[mask]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def q_props(qprecond, **kw):
    d = dict(qprecond=qprecond, qmaxiters=4000, qepsilon=1e-10, resnorm=1.0, dt=10.0)
    d.update(kw)
    return SolverProps(**d)


def h_props(hprecond, **kw):
    d = dict(hprecond=hprecond, maxiters=4000, epsilon=1e-10, resnorm=1.0, dt=30.0, theta=0.55)
    d.update(kw)
    return SolverProps(**d)


def stopping_ratio(oracle, prob, q, qprecond):
    """sqrt(eps/eps0) of CGSolveQ's stopping rule (main/phys.c:2470-2524) for the
    solution q, evaluated on the CPU with the oracle's own operators: the
    scaled residual for qprecond 1, the plain residual for 0 and 2."""
    import numpy as np
    g = prob.grid
    m = g.active_mask()
    if qprecond == 1:
        c = oracle.condition_q(g, prob.D, np.ones(g.n3))
        coef, fcoef = oracle.qcoefficients(g, prob.D, c, 1)
        b = np.where(m, prob.src / c, 0.0)

        def res(x):
            return b - oracle.operator_qc(g, coef, fcoef, np.where(m, x * c, 0.0))
    else:
        coef, _ = oracle.qcoefficients(g, prob.D, np.ones(g.n3), 0)

        def res(x):
            return prob.src - oracle.operator_q(g, prob.D, coef, np.where(m, x, 0.0) + np.where(m, 0.0, prob.q))
    r, r0 = res(q)[m], res(prob.q)[m]
    return float(np.linalg.norm(r) / np.linalg.norm(r0))
