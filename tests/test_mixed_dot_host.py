"""Accuracy of the batched mixed-precision solver's inner products (CPU).

The kernel accumulates each thread's share of p.Ap, r.r and r.M^-1 r in
double-float on the FP32 pipe (suntans_gb300/csrc/sgpu_batch.cu, df_addprod):
TwoProduct by one FMA, TwoSum of the high words, the errors gathered in the
low word -- the Dot2 scheme of Ogita, Rump and Oishi ("Accurate sum and dot
product", SIAM J. Sci. Comput. 26, 2005) -- and combines the thread partials in
FP64.  Its published bound for n terms is
    |dot2 - x.y| <= u |x.y| + gamma_n^2 sum|x_i y_i|,  u = 2^-24,
    gamma_n = n u / (1 - n u),
where the final u|x.y| becomes 2^-53 |x.y| here because the pair is added in
FP64.  Restated below with numpy's IEEE FP32 arithmetic (the exact product
and its FMA remainder formed in FP64, where a product of two floats is exact)
on the FP32 residual of a stiff seeded grid, split over threads as the kernel
splits a 39.7M-unknown instance (~340 terms per thread): the error stays
within the bound, and below the worst-case error of plain sequential FP64
accumulation over the same terms."""
import math

import numpy as np

from oracle.oracle import Oracle
from tests._cases import grid_cases
from suntans_gb300 import gridgen as gg

U32 = 2.0 ** -24


def df_dot(x, y):
    """One thread's double-float accumulation (df_addprod), value as FP64."""
    hi = np.float32(0.0)
    lo = np.float32(0.0)
    for a, b in zip(x, y):
        p = np.float32(a * b)
        e = np.float32(np.float64(a) * np.float64(b) - np.float64(p))
        t = np.float32(hi + p)
        bp = np.float32(t - hi)
        err = np.float32(np.float32(hi - np.float32(t - bp)) + np.float32(p - bp))
        hi = t
        lo = np.float32(lo + np.float32(err + e))
    return float(hi) + float(lo)


def test_double_float_dot_within_published_bound():
    g = dict(grid_cases())["tri3000_partial"]()
    prob = gg.make_q_problem(g, seed=1, q0_sigma=0.01)
    o = Oracle("port")
    coef, _ = o.qcoefficients(g, prob.D, np.ones(g.n3), 0)
    m = g.active_mask()
    r = (prob.src - o.operator_q(g, prob.D, coef, np.where(m, prob.q, 0.0)))[m]
    x = r.astype(np.float32)
    rng = np.random.default_rng(3)
    y = (x * (1 + 1e-3 * rng.standard_normal(x.size))).astype(np.float32)  # a p.z-like pair
    n_t = 340
    for a, b in ((x, x), (x, y)):
        exact = math.fsum(float(np.float64(u) * np.float64(v)) for u, v in zip(a, b))
        parts = [df_dot(a[i:i + n_t], b[i:i + n_t]) for i in range(0, a.size, n_t)]
        got = math.fsum(parts)  # the kernel adds thread partials in FP64 (a fixed tree)
        s_abs = math.fsum(abs(float(np.float64(u) * np.float64(v))) for u, v in zip(a, b))
        gam = n_t * U32 / (1 - n_t * U32)
        bound = 2.0 ** -53 * abs(exact) + gam ** 2 * s_abs + len(parts) * 2.0 ** -53 * s_abs
        assert abs(got - exact) <= bound, (got, exact, bound)
        # worst case of plain sequential FP64 accumulation over the same terms
        assert abs(got - exact) <= a.size * 2.0 ** -53 * s_abs
