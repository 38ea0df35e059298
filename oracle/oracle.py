"""ctypes bindings to the CPU oracles -- TEST INFRASTRUCTURE ONLY.

Two libraries share one flat-array interface (cg_oracle.h):

* ``port``  oracle/_build/libsgo_port.so, the plain-C restatement of the
  reference algorithm (cg_oracle.c); built on any host by ``make -C oracle port``.
* ``ref``   oracle/_ref/libsuntans_ref.so, the reference's own main/phys.c
  compiled from its sources (ref_harness.c); exists only where the reference
  tree was present at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libsgo_port.so")
REF_SO = os.path.join(HERE, "_ref", "libsuntans_ref.so")

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class SgoGrid(C.Structure):
    _fields_ = [("Nc", C.c_int), ("Ne", C.c_int), ("maxfaces", C.c_int), ("Nkmax", C.c_int),
                ("nfaces", _ip), ("neigh", _ip), ("face", _ip), ("Nk", _ip), ("Nke", _ip),
                ("ctop", _ip), ("cellp", _ip), ("celldist", _ip),
                ("Ac", _dp), ("df", _dp), ("dg", _dp), ("dzz", _dp), ("dzf", _dp)]


class SgoProp(C.Structure):
    _fields_ = [("qprecond", C.c_int), ("qmaxiters", C.c_int), ("qepsilon", C.c_double),
                ("hprecond", C.c_int), ("maxiters", C.c_int), ("epsilon", C.c_double),
                ("resnorm", C.c_double), ("grav", C.c_double), ("theta", C.c_double),
                ("dt", C.c_double)]


class SgoExt(C.Structure):
    _fields_ = [("normal", _ip), ("grad", _ip), ("edgep", _ip), ("edgedist", _ip), ("etop", _ip)]


class SgoVgrid(C.Structure):
    _fields_ = [("dz", _dp), ("dv", _dp), ("dzbot", _dp), ("Nkc", _ip), ("smoothbot", C.c_double),
                ("dzsmall", C.c_double)]


class SgoUpred(C.Structure):
    _fields_ = [("u", _dp), ("w", _dp), ("tau_T", _dp), ("CdT", _dp), ("CdB", _dp), ("nu_tv", _dp),
                ("nu_lax", _dp), ("nu", C.c_double), ("laxWendroff_Vertical", C.c_double),
                ("thetaM", C.c_double), ("nonlinear", C.c_int)]


class SgoUbnd(C.Structure):
    _fields_ = [("edgep", _ip), ("edgedist", _ip), ("mark", _ip), ("n1", _dp), ("n2", _dp)]


class SgoWpred(C.Structure):
    _fields_ = [("q", _dp), ("nu_tv", _dp), ("nu_lax", _dp), ("utmp2", _dp), ("nu", C.c_double),
                ("nu_H", C.c_double), ("CdW", C.c_double), ("laxWendroff_Vertical", C.c_double),
                ("nonlinear", C.c_int), ("conserveMomentum", C.c_int), ("n", C.c_int), ("AB", C.c_int)]


class SgoResult(C.Structure):
    _fields_ = [("niters", C.c_int), ("eps", C.c_double), ("eps0", C.c_double),
                ("t_setup", C.c_double), ("t_loop", C.c_double)]


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


def _make_args() -> list:
    env = os.environ.get("SUNTANS_REFDIR")
    return [f"REFDIR={env}"] if env else []


def build_ref() -> Optional[str]:
    """Builds oracle/_ref from the reference's main/ sources: SUNTANS_REFDIR
    when set, else the Makefile's default location; None where they are absent."""
    chk = subprocess.run(["make", "-s", "-C", HERE, "refcheck", *_make_args()], capture_output=True)
    if chk.returncode != 0:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", *_make_args()], check=True)
    return REF_SO


def ref_dir() -> Optional[str]:
    """The reference's main/ directory: SUNTANS_REFDIR when set, else the one
    oracle/_ref was built from (recorded by the Makefile); None on hosts
    without the reference sources (the GPU machine)."""
    d = os.environ.get("SUNTANS_REFDIR")
    if not d:
        rec = os.path.join(HERE, "_ref", "refdir.txt")
        if not os.path.isfile(rec):
            build_ref()  # writes the record where the sources are present
        if os.path.isfile(rec):
            d = open(rec).read().strip()
    return d if d and os.path.isfile(os.path.join(d, "phys.c")) else None


def ref_examples_dir() -> Optional[str]:
    """The reference's examples/ directory, beside main/ (None where absent)."""
    d = ref_dir()
    return os.path.join(os.path.dirname(d), "examples") if d else None


class Oracle:
    """One of the two oracle libraries, with numpy-level wrappers."""

    def __init__(self, which: str = "port"):
        path = PORT_SO if which == "port" else REF_SO
        if which == "port" and not os.path.exists(path):
            build_port()
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.prefix = "sgo_" if which == "port" else "ref_"
        self.which = which

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    @staticmethod
    def _grid(g):
        keep = [np.ascontiguousarray(x) for x in
                (g.nfaces, g.neigh, g.face, g.Nk, g.Nke, g.ctop, g.cellp, g.celldist,
                 g.Ac, g.df, g.dg, g.dzz, g.dzf)]
        s = SgoGrid(g.Nc, g.Ne, g.maxfaces, g.Nkmax,
                    *[_ptr(x, _ip) for x in keep[:8]], *[_ptr(x, _dp) for x in keep[8:]])
        return s, keep

    @staticmethod
    def _prop(p):
        return SgoProp(p.qprecond, p.qmaxiters, p.qepsilon, p.hprecond, p.maxiters, p.epsilon,
                       float(p.resnorm), p.grav, p.theta, p.dt)

    def cgsolveq(self, prob, props):
        """Runs CGSolveQ on copies of prob.q / prob.src / prob.c; returns (q, niters)."""
        g = prob.grid
        s, keep = self._grid(g)
        q = np.array(prob.q, dtype=np.float64, copy=True)
        src = np.array(prob.src, dtype=np.float64, copy=True)
        c = np.array(prob.c, dtype=np.float64, copy=True)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        pr = self._prop(props)
        res = SgoResult()
        self._fn("cgsolveq")(C.byref(s), _ptr(D, _dp), _ptr(q, _dp), _ptr(src, _dp), _ptr(c, _dp),
                             C.byref(pr), C.byref(res))
        return q, int(res.niters)

    def cgsolve(self, prob, props):
        """Runs CGSolve on copies of prob.h / prob.htmp; returns (h, niters)."""
        g = prob.grid
        s, keep = self._grid(g)
        h = np.array(prob.h, dtype=np.float64, copy=True)
        htmp = np.array(prob.htmp, dtype=np.float64, copy=True)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        pr = self._prop(props)
        res = SgoResult()
        self._fn("cgsolve")(C.byref(s), _ptr(D, _dp), _ptr(h, _dp), _ptr(htmp, _dp), C.byref(pr),
                            C.byref(res))
        return h, int(res.niters)

    def cgsolveq_timed(self, prob, props):
        """cgsolveq plus the port's own timing: (q, niters, seconds before the
        iteration loop, seconds in it).  Port only."""
        assert self.which == "port"
        g = prob.grid
        s, keep = self._grid(g)
        q = np.array(prob.q, dtype=np.float64, copy=True)
        src = np.array(prob.src, dtype=np.float64, copy=True)
        c = np.array(prob.c, dtype=np.float64, copy=True)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        pr = self._prop(props)
        res = SgoResult()
        self._fn("cgsolveq")(C.byref(s), _ptr(D, _dp), _ptr(q, _dp), _ptr(src, _dp), _ptr(c, _dp),
                             C.byref(pr), C.byref(res))
        return q, int(res.niters), float(res.t_setup), float(res.t_loop)

    def cgsolve_timed(self, prob, props):
        """cgsolve plus the port's own timing: (h, niters, setup s, loop s).  Port only."""
        assert self.which == "port"
        g = prob.grid
        s, keep = self._grid(g)
        h = np.array(prob.h, dtype=np.float64, copy=True)
        htmp = np.array(prob.htmp, dtype=np.float64, copy=True)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        pr = self._prop(props)
        res = SgoResult()
        self._fn("cgsolve")(C.byref(s), _ptr(D, _dp), _ptr(h, _dp), _ptr(htmp, _dp), C.byref(pr), C.byref(res))
        return h, int(res.niters), float(res.t_setup), float(res.t_loop)

    def iteration_span(self, prob, props, solver="q"):
        """Iteration counts of the port's solve with the reference's sequential
        inner products and with pairwise ones: (sequential, pairwise).  A
        parallel reduction adds in neither order; on an ill-conditioned system
        the iteration at which the residual crosses the tolerance moves with
        that order alone (the solution stays within round-off of the
        reference's).  Port only."""
        assert self.which == "port"
        fn = self.cgsolveq if solver == "q" else self.cgsolve
        n_seq = fn(prob, props)[1]
        self.lib.sgo_set_sum_order(1)
        try:
            n_pair = fn(prob, props)[1]
        finally:
            self.lib.sgo_set_sum_order(0)
        return n_seq, n_pair

    # ---- operator pieces ----
    def qcoefficients(self, g, D, c, qprecond):
        s, keep = self._grid(g)
        coef = np.zeros(g.n3)
        fcoef = np.zeros(g.n3 * g.maxfaces)
        c = np.ascontiguousarray(c, dtype=np.float64)
        D = np.ascontiguousarray(D, dtype=np.float64)
        self._fn("qcoefficients")(C.byref(s), _ptr(D, _dp), _ptr(c, _dp), C.c_int(qprecond),
                                  _ptr(coef, _dp), _ptr(fcoef, _dp))
        return coef, fcoef

    def operator_q(self, g, D, coef, x, y0=None):
        s, keep = self._grid(g)
        y = np.zeros(g.n3) if y0 is None else np.array(y0, copy=True)
        D = np.ascontiguousarray(D, dtype=np.float64)
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._fn("operator_q")(C.byref(s), _ptr(D, _dp), _ptr(coef, _dp), _ptr(x, _dp), _ptr(y, _dp))
        return y

    def operator_qc(self, g, coef, fcoef, x, y0=None):
        s, keep = self._grid(g)
        y = np.zeros(g.n3) if y0 is None else np.array(y0, copy=True)
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        fcoef = np.ascontiguousarray(fcoef, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._fn("operator_qc")(C.byref(s), _ptr(coef, _dp), _ptr(fcoef, _dp), _ptr(x, _dp), _ptr(y, _dp))
        return y

    def condition_q(self, g, D, c0=None):
        s, keep = self._grid(g)
        c = np.ones(g.n3) if c0 is None else np.array(c0, copy=True)
        D = np.ascontiguousarray(D, dtype=np.float64)
        self._fn("condition_q")(C.byref(s), _ptr(D, _dp), _ptr(c, _dp))
        return c

    def preconditioner(self, g, coef, x, xc0=None):
        s, keep = self._grid(g)
        xc = np.zeros(g.n3) if xc0 is None else np.array(xc0, copy=True)
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._fn("preconditioner")(C.byref(s), _ptr(coef, _dp), _ptr(x, _dp), _ptr(xc, _dp))
        return xc

    def hcoefficients(self, g, D, props):
        s, keep = self._grid(g)
        hcoef = np.zeros(g.Nc)
        hfcoef = np.zeros(g.Nc * g.maxfaces)
        D = np.ascontiguousarray(D, dtype=np.float64)
        pr = self._prop(props)
        self._fn("hcoefficients")(C.byref(s), _ptr(D, _dp), C.byref(pr), _ptr(hcoef, _dp), _ptr(hfcoef, _dp))
        return hcoef, hfcoef

    def operator_h(self, g, hcoef, hfcoef, x, y0=None):
        s, keep = self._grid(g)
        y = np.zeros(g.Nc) if y0 is None else np.array(y0, copy=True)
        hcoef = np.ascontiguousarray(hcoef, dtype=np.float64)
        hfcoef = np.ascontiguousarray(hfcoef, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._fn("operator_h")(C.byref(s), _ptr(hcoef, _dp), _ptr(hfcoef, _dp), _ptr(x, _dp), _ptr(y, _dp))
        return y


    # ---- the steps around CGSolveQ ----
    @staticmethod
    def _ext(st):
        g = st.grid
        keep = [np.ascontiguousarray(x, dtype=np.int32) for x in (g.normal, g.grad, st.edgep, st.edgedist, st.etop)]
        return SgoExt(*[_ptr(x, _ip) for x in keep]), keep

    def compute_qsource(self, st, props):
        """ComputeQSource on the step fields st; returns (src, D)."""
        g = st.grid
        s, keep = self._grid(g)
        x, keepx = self._ext(st)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (st.u, st.utmp2, st.w, st.wtmp2)]
        src = np.zeros(g.n3)
        D = np.zeros(max(g.Ne, 1))
        pr = self._prop(props)
        self._fn("compute_qsource")(C.byref(s), C.byref(x), *[_ptr(a, _dp) for a in arrs], C.byref(pr),
                                    _ptr(src, _dp), _ptr(D, _dp))
        return src, D[:g.Ne]

    def corrector(self, st, qc, D, props):
        """Corrector with the correction qc; returns (u, w, q) updated copies of st's."""
        g = st.grid
        s, keep = self._grid(g)
        x, keepx = self._ext(st)
        qc = np.ascontiguousarray(qc, dtype=np.float64)
        D = np.ascontiguousarray(D, dtype=np.float64)
        u = np.array(st.u, dtype=np.float64, copy=True)
        w = np.array(st.w, dtype=np.float64, copy=True)
        q = np.array(st.q, dtype=np.float64, copy=True)
        pr = self._prop(props)
        self._fn("corrector")(C.byref(s), C.byref(x), _ptr(qc, _dp), _ptr(D, _dp), C.byref(pr), _ptr(u, _dp),
                              _ptr(w, _dp), _ptr(q, _dp))
        return u, w, q


    # ---- the vertical grid of the step ----
    @staticmethod
    def _vgrid(vf):
        g = vf.grid
        keep = [np.ascontiguousarray(g.dz, dtype=np.float64), np.ascontiguousarray(g.dv, dtype=np.float64),
                np.ascontiguousarray(vf.dzbot, dtype=np.float64), np.ascontiguousarray(vf.Nkc, dtype=np.int32)]
        return SgoVgrid(_ptr(keep[0], _dp), _ptr(keep[1], _dp), _ptr(keep[2], _dp), _ptr(keep[3], _ip),
                        vf.smoothbot, vf.dzsmall), keep

    def _vext(self, vf, etop):
        g = vf.grid
        keep = [np.ascontiguousarray(g.normal, dtype=np.int32), np.ascontiguousarray(g.grad, dtype=np.int32),
                np.zeros(1, np.int32), np.zeros(2, np.int32), etop]
        return SgoExt(*[_ptr(x, _ip) for x in keep]), keep

    def update_dz(self, vf, linearFS=0):
        """UpdateDZ(option 0): returns (ctop, etop, dzz, ctopold, etopold, dzzold)."""
        g = vf.grid
        s, keep = self._grid(g)
        v, keepv = self._vgrid(vf)
        ctop = np.array(vf.ctop, dtype=np.int32, copy=True)
        etop = np.array(vf.etop, dtype=np.int32, copy=True)
        x, keepx = self._vext(vf, etop)
        dzz = np.array(vf.dzz, dtype=np.float64, copy=True)
        ctopold = np.full(g.Nc, -7, dtype=np.int32)
        etopold = np.full(max(g.Ne, 1), -7, dtype=np.int32)
        dzzold = np.full(g.n3, -7.0)
        h = np.ascontiguousarray(vf.h, dtype=np.float64)
        self._fn("update_dz")(C.byref(s), C.byref(x), C.byref(v), _ptr(h, _dp), C.c_int(linearFS),
                              _ptr(ctop, _ip), _ptr(etop, _ip), _ptr(dzz, _dp), _ptr(ctopold, _ip),
                              _ptr(etopold, _ip), _ptr(dzzold, _dp))
        return ctop, etop[:g.Ne], dzz, ctopold, etopold[:g.Ne], dzzold

    def set_flux_height(self, vf, dzz=None, etop=None):
        """SetFluxHeight: returns (dzf rows of Nkc levels, dzz after the smoothbot adjustments)."""
        g = vf.grid
        s, keep = self._grid(g)
        v, keepv = self._vgrid(vf)
        et = np.array(vf.etop if etop is None else etop, dtype=np.int32, copy=True)
        x, keepx = self._vext(vf, et)
        dzz = np.array(vf.dzz if dzz is None else dzz, dtype=np.float64, copy=True)
        dzf = np.full(int(np.sum(vf.Nkc)), -7.0)
        h = np.ascontiguousarray(vf.h, dtype=np.float64)
        u = np.ascontiguousarray(vf.u, dtype=np.float64)
        self._fn("set_flux_height")(C.byref(s), C.byref(x), C.byref(v), _ptr(h, _dp), _ptr(u, _dp), _ptr(dzz, _dp),
                                    _ptr(dzf, _dp))
        return dzf, dzz


    # ---- UPredictor (main/phys.c:2579-3077) ----
    @staticmethod
    def _upred(uf):
        keep = [np.ascontiguousarray(a, dtype=np.float64)
                for a in (uf.u, uf.w, uf.tau_T, uf.CdT, uf.CdB, uf.nu_tv, uf.nu_lax)]
        return SgoUpred(*[_ptr(a, _dp) for a in keep], uf.nu, uf.laxWendroff_Vertical, uf.thetaM,
                        uf.nonlinear), keep

    @staticmethod
    def _ubnd(uf):
        ki = [np.ascontiguousarray(a, dtype=np.int32) for a in (uf.bedgep, uf.bedgedist, uf.mark)]
        kd = [np.ascontiguousarray(a, dtype=np.float64) for a in (uf.n1, uf.n2)]
        return SgoUbnd(*[_ptr(a, _ip) for a in ki], *[_ptr(a, _dp) for a in kd]), ki + kd

    @staticmethod
    def _uext(uf, etop):
        g = uf.grid
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (g.normal, g.grad, uf.edgep, uf.edgedist, etop)]
        return SgoExt(*[_ptr(x, _ip) for x in keep]), keep

    def upredictor_vertical(self, uf, props, grid=None, etop=None):
        """U***, E, D on the computational edges; returns (utmp, E, D, NaN count)."""
        g = uf.grid if grid is None else grid
        s, keep = self._grid(g)
        x, kx = self._uext(uf, uf.etop if etop is None else etop)
        up, ku = self._upred(uf)
        h = np.ascontiguousarray(uf.h, dtype=np.float64)
        utmp = np.array(uf.utmp, dtype=np.float64, copy=True)
        E = np.zeros(max(int(g.Nke.sum()), 1))
        D = np.full(max(g.Ne, 1), -7.0)
        pr = self._prop(props)
        n = self._fn("upredictor_vertical")(C.byref(s), C.byref(x), C.byref(up), _ptr(h, _dp), C.byref(pr),
                                            _ptr(utmp, _dp), _ptr(E, _dp), _ptr(D, _dp))
        return utmp, E[:int(g.Nke.sum())], D[:g.Ne], int(n)

    def upredictor_rhs(self, uf, props, utmp, h=None, grid=None, etop=None):
        """The free-surface right-hand side on computational cells (others left 0)."""
        g = uf.grid if grid is None else grid
        s, keep = self._grid(g)
        x, kx = self._uext(uf, uf.etop if etop is None else etop)
        up, ku = self._upred(uf)
        hh = np.ascontiguousarray(uf.h if h is None else h, dtype=np.float64)
        ut = np.ascontiguousarray(utmp, dtype=np.float64)
        htmp = np.zeros(g.Nc)
        pr = self._prop(props)
        self._fn("upredictor_rhs")(C.byref(s), C.byref(x), C.byref(up), _ptr(hh, _dp), C.byref(pr), _ptr(ut, _dp),
                                   _ptr(htmp, _dp))
        return htmp

    def upredictor_velocity(self, uf, vf, props, utmp, E, h, u=None, grid=None, etop=None):
        """Dry-cell clip and u on the computational edges; returns (h, active, u)."""
        g = uf.grid if grid is None else grid
        s, keep = self._grid(g)
        x, kx = self._uext(uf, uf.etop if etop is None else etop)
        v, kv = self._vgrid(vf)
        ut = np.ascontiguousarray(utmp, dtype=np.float64)
        EE = np.ascontiguousarray(E, dtype=np.float64)
        hh = np.array(h, dtype=np.float64, copy=True)
        active = np.full(g.Nc, 7, dtype=np.uint8)
        uu = np.array(uf.u if u is None else u, dtype=np.float64, copy=True)
        pr = self._prop(props)
        self._fn("upredictor_velocity")(C.byref(s), C.byref(x), C.byref(v), C.byref(pr), _ptr(ut, _dp),
                                        _ptr(EE, _dp), _ptr(hh, _dp),
                                        active.ctypes.data_as(C.POINTER(C.c_ubyte)), _ptr(uu, _dp))
        return hh, active, uu

    def upredictor_boundary(self, uf, utmp, u, grid=None, etop=None):
        """u on type-2 edges and on the mark-3 faces of type-3 cells."""
        g = uf.grid if grid is None else grid
        s, keep = self._grid(g)
        x, kx = self._uext(uf, uf.etop if etop is None else etop)
        b, kb = self._ubnd(uf)
        ut = np.ascontiguousarray(utmp, dtype=np.float64)
        uu = np.array(u, dtype=np.float64, copy=True)
        self._fn("upredictor_boundary")(C.byref(s), C.byref(x), C.byref(b), _ptr(ut, _dp), _ptr(uu, _dp))
        return uu

    def upredictor(self, uf, vf, props):
        """The whole UPredictor with CGSolve, from the grid's ctop / dzz and
        uf.etop; returns a dict of u, h, utmp, E, D, ctop, etop, dzz, active,
        niters and the NaN count."""
        g = uf.grid
        s, keep = self._grid(g)
        ctop = np.array(g.ctop, dtype=np.int32, copy=True)
        etop = np.array(uf.etop, dtype=np.int32, copy=True)
        dzz = np.array(g.dzz, dtype=np.float64, copy=True)
        x, kx = self._uext(uf, etop)
        x.etop = _ptr(etop, _ip)
        v, kv = self._vgrid(vf)
        up, ku = self._upred(uf)
        b, kb = self._ubnd(uf)
        u = np.array(uf.u, dtype=np.float64, copy=True)
        h = np.array(uf.h, dtype=np.float64, copy=True)
        utmp = np.array(uf.utmp, dtype=np.float64, copy=True)
        E = np.zeros(max(int(g.Nke.sum()), 1))
        D = np.zeros(max(g.Ne, 1))
        active = np.full(g.Nc, 7, dtype=np.uint8)
        res = SgoResult()
        pr = self._prop(props)
        n = self._fn("upredictor")(C.byref(s), C.byref(x), C.byref(v), C.byref(up), C.byref(b), C.byref(pr),
                                   _ptr(u, _dp), _ptr(h, _dp), _ptr(utmp, _dp), _ptr(E, _dp), _ptr(D, _dp),
                                   _ptr(ctop, _ip), _ptr(etop, _ip), _ptr(dzz, _dp),
                                   active.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(res))
        return dict(u=u, h=h, utmp=utmp, E=E[:int(g.Nke.sum())], D=D[:g.Ne], ctop=ctop, etop=etop, dzz=dzz,
                    active=active, niters=res.niters, nnan=int(n))

    # ---- WPredictor (main/phys.c:2025-2287) ----
    def wpredictor(self, wf, props):
        """Returns (w, Cn_W, Cn_W2) after one WPredictor."""
        g = wf.grid
        s, keep = self._grid(g)
        x, kx = self._uext(wf, wf.etop)
        kd = [np.ascontiguousarray(a, dtype=np.float64) for a in (wf.q, wf.nu_tv, wf.nu_lax, wf.utmp2)]
        wp = SgoWpred(*[_ptr(a, _dp) for a in kd], wf.nu, wf.nu_H, wf.CdW, wf.laxWendroff_Vertical, wf.nonlinear,
                      wf.conserveMomentum, wf.n, wf.AB)
        w = np.array(wf.w, dtype=np.float64, copy=True)
        cw = np.array(wf.Cn_W, dtype=np.float64, copy=True)
        cw2 = np.array(wf.Cn_W2, dtype=np.float64, copy=True)
        pr = self._prop(props)
        rc = self._fn("wpredictor")(C.byref(s), C.byref(x), C.byref(wp), C.byref(pr), _ptr(w, _dp), _ptr(cw, _dp),
                                    _ptr(cw2, _dp))
        if rc != 0:
            raise ValueError("wpredictor: unsupported settings")
        return w, cw, cw2

    # ---- the reference's grid reader and field writers (ref library only) ----
    def read_grid(self, datadir: str) -> dict:
        """ReadGrid (main/gridio.c:54-187) on a folder holding suntans.dat and
        the grid files; returns the gridT arrays by name."""
        if self.which != "ref":
            raise RuntimeError("read_grid needs the reference library")
        sizes = np.zeros(6, dtype=np.int32)
        self.lib.ref_read_grid(datadir.encode(), _ptr(sizes, _ip))
        Nc, Ne, Np, mf, Nkmax, nneigh = (int(x) for x in sizes)
        out = {"Nc": Nc, "Ne": Ne, "Np": Np, "maxfaces": mf, "Nkmax": Nkmax, "Nneighs": nneigh}
        self.lib.ref_grid_ints.restype = C.c_long
        self.lib.ref_grid_dbls.restype = C.c_long
        cap = max(16, 8 * (Nc * mf + 2 * Ne + 8 * Np + Nkmax + 16))
        for name in ("nfaces", "Nk", "mnptr", "cellp", "face", "neigh", "normal", "cells", "Nke", "Nkc",
                     "mark", "edge_id", "eptr", "edgep", "grad", "gradf", "celldist", "edgedist",
                     "localtoglobalpoints", "numppneighs", "numpeneighs", "numpcneighs", "Nkp", "edges",
                     "ppneighs", "peneighs", "pcneighs"):
            buf = np.zeros(cap, dtype=np.int32)
            n = self.lib.ref_grid_ints(name.encode(), _ptr(buf, _ip))
            out[name] = buf[:n].copy()
        for name in ("xv", "yv", "Ac", "dv", "def", "df", "dg", "n1", "n2", "xe", "ye", "xp", "yp", "dz",
                     "Actotal"):
            buf = np.zeros(cap, dtype=np.float64)
            n = self.lib.ref_grid_dbls(name.encode(), _ptr(buf, _dp))
            out[name] = buf[:n].copy()
        return out

    def read_main_grid(self, datadir: str) -> dict:
        """ReadMainGrid (main/gridio.c:256-266) after InitMainGrid, on a folder
        holding suntans.dat and the points / edges / cells files; returns the
        gridT arrays it fills by name (cells and neigh whole: maxfaces per
        cell, slots past nfaces as the reference left them)."""
        if self.which != "ref":
            raise RuntimeError("read_main_grid needs the reference library")
        sizes = np.zeros(6, dtype=np.int32)
        self.lib.ref_read_main_grid(datadir.encode(), _ptr(sizes, _ip))
        Nc, Ne, Np, mf = (int(x) for x in sizes[:4])
        out = {"Nc": Nc, "Ne": Ne, "Np": Np, "maxfaces": mf}
        self.lib.ref_grid_ints.restype = C.c_long
        self.lib.ref_grid_dbls.restype = C.c_long
        cap = max(16, Nc * mf + 2 * Ne + Np + 16)
        for name in ("nfaces", "cells", "neigh", "mark", "edge_id", "grad", "edges"):
            buf = np.zeros(cap, dtype=np.int32)
            n = self.lib.ref_grid_ints(name.encode(), _ptr(buf, _ip))
            out[name] = buf[:n].copy()
        for name in ("xv", "yv", "xp", "yp"):
            buf = np.zeros(cap, dtype=np.float64)
            n = self.lib.ref_grid_dbls(name.encode(), _ptr(buf, _dp))
            out[name] = buf[:n].copy()
        return out

    def write_2d(self, path: str, x) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.lib.ref_write_2d(path.encode(), C.c_int(x.size), _ptr(x, _dp))

    def write_3d(self, path: str, Nk, Nkmax: int, flat, extra: int = 0) -> None:
        Nk = np.ascontiguousarray(Nk, dtype=np.int32)
        flat = np.ascontiguousarray(flat, dtype=np.float64)
        self.lib.ref_write_3d(path.encode(), C.c_int(Nk.size), C.c_int(Nkmax), _ptr(Nk, _ip), _ptr(flat, _dp),
                              C.c_int(extra))


def available(which: str) -> bool:
    return os.path.exists(PORT_SO if which == "port" else REF_SO)
