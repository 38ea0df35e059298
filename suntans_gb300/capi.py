"""ctypes binding of the C ABI in include/suntans_gb300.h.

The library is the in-tree build suntans_gb300/_lib/libsuntans_gb300.so.
Loading fails loudly (ImportError) when it is missing; there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .grid import SunGrid, SolverProps

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsuntans_gb300.so")

# status codes, include/suntans_gb300.h
OK, MAXITER, BREAKDOWN, TIMEOUT, OOM, BAD_GRID, BAD_ARG, CUDA_ERROR, NO_DEVICE = range(9)

# every symbol the header declares
EXPORTS = [
    "sgpu_create", "sgpu_destroy", "sgpu_last_error", "sgpu_status_string",
    "sgpu_cgsolveq", "sgpu_cgsolve",
    "sgpu_q_upload", "sgpu_q_solve", "sgpu_q_download",
    "sgpu_h_upload", "sgpu_h_solve", "sgpu_h_download",
    "sgpu_set_timeout_ns", "sgpu_set_grid", "sgpu_stream", "sgpu_phase_times",
    "sgpu_cgsolve_noalloc",
    "sgpu_step_grid", "sgpu_compute_qsource", "sgpu_corrector", "sgpu_pressure_step", "sgpu_nonhydrostatic_step",
    "sgpu_update_dz", "sgpu_set_flux_height",
    "sgpu_wpredictor",
    "sgpu_upredictor_grid", "sgpu_upredictor_vertical", "sgpu_upredictor_rhs", "sgpu_upredictor_finish",
    "sgpu_upredictor",
    "sgpu_batch_create", "sgpu_batch_destroy", "sgpu_batch_last_error", "sgpu_batch_bytes_per_request",
    "sgpu_batch_add", "sgpu_batch_run", "sgpu_batch_launch", "sgpu_batch_wait", "sgpu_batch_state", "sgpu_batch_result", "sgpu_batch_set", "sgpu_batch_set_tile_slots", "sgpu_batch_set_fusion", "sgpu_batch_set_stride",
    "sgpu_batch_stream", "sgpu_batch_phase_times", "sgpu_batch_resubmit", "sgpu_batch_use_graph",
    "sgpu_batch_graph_launches",
]
TOO_LARGE = 9

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_dpp = C.POINTER(C.c_void_p)


class GridDesc(C.Structure):
    _fields_ = [("Nc", C.c_int), ("Ne", C.c_int), ("maxfaces", C.c_int), ("Nkmax", C.c_int),
                ("nfaces", _ip), ("neigh", _ip), ("face", _ip), ("Nk", _ip), ("Nke", _ip),
                ("cellp", _ip), ("celldist", _ip), ("Ac", _dp), ("df", _dp), ("dg", _dp)]


class Props(C.Structure):
    _fields_ = [("qprecond", C.c_int), ("qmaxiters", C.c_int), ("qepsilon", C.c_double),
                ("hprecond", C.c_int), ("maxiters", C.c_int), ("epsilon", C.c_double),
                ("resnorm", C.c_double), ("grav", C.c_double), ("theta", C.c_double),
                ("dt", C.c_double)]


class NoallocGrid(C.Structure):
    """sgpu_noalloc_grid: sizes plus DEVICE pointers (integers) owned by the caller."""
    _fields_ = [("Nc", C.c_int), ("Ne", C.c_int), ("maxfaces", C.c_int), ("ncomp", C.c_int),
                ("cellp", C.c_void_p), ("nfaces", C.c_void_p), ("neigh", C.c_void_p), ("face", C.c_void_p),
                ("Ac", C.c_void_p), ("df", C.c_void_p), ("dg", C.c_void_p)]


class VGrid(C.Structure):
    _fields_ = [("dz", _dp), ("dv", _dp), ("dzbot", _dp), ("Nkc", _ip), ("smoothbot", C.c_double),
                ("dzsmall", C.c_double)]


class UPredFieldsC(C.Structure):
    _fields_ = [("u", _dpp), ("w", _dpp), ("nu_tv", _dpp), ("nu_lax", _dpp), ("tau_T", _dp), ("CdT", _dp),
                ("CdB", _dp), ("nu", C.c_double), ("laxWendroff_Vertical", C.c_double), ("thetaM", C.c_double),
                ("nonlinear", C.c_int)]


class WPredFieldsC(C.Structure):
    _fields_ = [("q", _dpp), ("nu_tv", _dpp), ("nu_lax", _dpp), ("utmp2", _dpp), ("nu", C.c_double),
                ("nu_H", C.c_double), ("CdW", C.c_double), ("laxWendroff_Vertical", C.c_double),
                ("nonlinear", C.c_int), ("conserveMomentum", C.c_int), ("n", C.c_int), ("AB", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("status", C.c_int), ("niters", C.c_int), ("eps", C.c_double), ("eps0", C.c_double),
                ("ms_solve", C.c_double), ("ms_total", C.c_double), ("unknowns", C.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library (raises ImportError if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (or python -m suntans_gb300.build)")
    lib = C.CDLL(LIB_PATH)
    lib.sgpu_create.argtypes = [C.POINTER(GridDesc), C.c_int, C.POINTER(C.c_void_p)]
    lib.sgpu_destroy.argtypes = [C.c_void_p]
    lib.sgpu_last_error.argtypes = [C.c_void_p]
    lib.sgpu_last_error.restype = C.c_char_p
    lib.sgpu_status_string.argtypes = [C.c_int]
    lib.sgpu_status_string.restype = C.c_char_p
    lib.sgpu_step_grid.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
    lib.sgpu_update_dz.argtypes = [C.c_void_p, C.POINTER(VGrid), _dp, C.c_int, _ip, _ip, _dpp, _ip, _ip, _dpp]
    lib.sgpu_set_flux_height.argtypes = [C.c_void_p, C.POINTER(VGrid), _ip, _dp, _dpp, _dpp, _dpp]
    _ucp = C.POINTER(C.c_ubyte)
    lib.sgpu_wpredictor.argtypes = [C.c_void_p, _ip, _dpp, C.POINTER(WPredFieldsC), C.POINTER(Props), _dpp, _dpp,
                                    _dpp]
    lib.sgpu_upredictor_grid.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _ip, _ip]
    lib.sgpu_upredictor_vertical.argtypes = [C.c_void_p, _ip, _ip, _dpp, _dpp, _dp, C.POINTER(UPredFieldsC),
                                             C.POINTER(Props), _dpp, _dpp, _dp]
    lib.sgpu_upredictor_rhs.argtypes = [C.c_void_p, _ip, _dpp, _dpp, _dpp, _dp, C.POINTER(Props), _dp]
    lib.sgpu_upredictor_finish.argtypes = [C.c_void_p, C.POINTER(VGrid), C.POINTER(Props), _ip, _ip, _dpp, _dpp,
                                           _dpp, _dp, _ucp, _dpp]
    lib.sgpu_upredictor.argtypes = [C.c_void_p, C.POINTER(VGrid), C.POINTER(UPredFieldsC), C.POINTER(Props), _ip,
                                    _ip, _dpp, _dpp, _dpp, _dp, _dpp, _dpp, _dp, _ucp, C.POINTER(Stats)]
    lib.sgpu_compute_qsource.argtypes = [C.c_void_p, _ip, _dpp, _dpp, _dpp, _dpp, _dpp, C.c_double, C.c_double,
                                         _dpp, _dp]
    lib.sgpu_corrector.argtypes = [C.c_void_p, _ip, _ip, _dpp, _dpp, _dp, C.c_double, _dpp, _dpp, _dpp]
    lib.sgpu_pressure_step.argtypes = [C.c_void_p, _ip, _ip, _dpp, _dpp, _dpp, _dpp, _dpp, _dpp, _dpp, _dpp, _dpp,
                                       C.POINTER(Props), C.POINTER(Stats)]
    lib.sgpu_nonhydrostatic_step.argtypes = [C.c_void_p, _ip, _ip, _dpp, _dpp, _dpp, _dpp, C.POINTER(WPredFieldsC),
                                             _dpp, _dpp, _dpp, _dpp, _dpp, _dpp, _dpp, C.POINTER(Props),
                                             C.POINTER(Stats)]
    lib.sgpu_cgsolveq.argtypes = [C.c_void_p, _ip, _dpp, _dpp, _dp, _dpp, _dpp, _dpp, C.POINTER(Props),
                                  C.POINTER(Stats)]
    lib.sgpu_cgsolve.argtypes = [C.c_void_p, _dp, _dp, _dp, C.POINTER(Props), C.POINTER(Stats)]
    lib.sgpu_q_upload.argtypes = [C.c_void_p, _ip, _dpp, _dpp, _dp, _dpp, _dpp, _dpp]
    lib.sgpu_q_solve.argtypes = [C.c_void_p, C.POINTER(Props), C.POINTER(Stats)]
    lib.sgpu_q_download.argtypes = [C.c_void_p, _dpp]
    lib.sgpu_h_upload.argtypes = [C.c_void_p, _dp, _dp, _dp]
    lib.sgpu_h_solve.argtypes = [C.c_void_p, C.POINTER(Props), C.POINTER(Stats)]
    lib.sgpu_h_download.argtypes = [C.c_void_p, _dp]
    lib.sgpu_set_timeout_ns.argtypes = [C.c_void_p, C.c_longlong]
    lib.sgpu_set_grid.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_stream.argtypes = [C.c_void_p]
    lib.sgpu_stream.restype = C.c_void_p
    lib.sgpu_cgsolve_noalloc.argtypes = [C.POINTER(NoallocGrid), C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.POINTER(Props), C.POINTER(Stats), C.c_void_p]
    lib.sgpu_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_longlong,
                                      C.c_int, C.POINTER(C.c_void_p)]
    lib.sgpu_batch_destroy.argtypes = [C.c_void_p]
    lib.sgpu_batch_last_error.argtypes = [C.c_void_p]
    lib.sgpu_batch_last_error.restype = C.c_char_p
    lib.sgpu_batch_bytes_per_request.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_longlong]
    lib.sgpu_batch_bytes_per_request.restype = C.c_longlong
    lib.sgpu_batch_add.argtypes = [C.c_void_p, C.POINTER(GridDesc), _ip, _dpp, _dpp, _dp, _dpp, _dpp, _dpp,
                                   C.c_double, C.c_int, C.c_double, C.POINTER(C.c_int)]
    lib.sgpu_batch_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                   C.POINTER(C.c_longlong)]
    lib.sgpu_batch_launch.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_batch_wait.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    lib.sgpu_batch_state.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_batch_result.argtypes = [C.c_void_p, C.c_int, _dpp, C.POINTER(Stats), C.c_int]
    lib.sgpu_batch_set.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_longlong]
    lib.sgpu_batch_set_tile_slots.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_batch_set_fusion.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_batch_set_stride.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.sgpu_batch_stream.argtypes = [C.c_void_p]
    lib.sgpu_batch_stream.restype = C.c_void_p
    lib.sgpu_batch_phase_times.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    lib.sgpu_phase_times.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    lib.sgpu_batch_resubmit.argtypes = [C.c_void_p, C.c_int, _dpp, C.c_double, C.c_int, C.c_int]
    lib.sgpu_batch_use_graph.argtypes = [C.c_void_p, C.c_int]
    lib.sgpu_batch_graph_launches.argtypes = [C.c_void_p]
    lib.sgpu_batch_graph_launches.restype = C.c_longlong
    _lib = lib
    return lib


def props_struct(p: SolverProps) -> Props:
    return Props(int(p.qprecond), int(p.qmaxiters), float(p.qepsilon), int(p.hprecond), int(p.maxiters),
                 float(p.epsilon), float(p.resnorm), float(p.grav), float(p.theta), float(p.dt))


def jagged(flat: np.ndarray, offsets: np.ndarray) -> np.ndarray:
    """Array of row pointers into a flat float64 buffer (the reference's REAL**)."""
    assert flat.dtype == np.float64 and flat.flags.c_contiguous
    return (flat.ctypes.data + 8 * offsets[:-1].astype(np.uint64)).astype(np.uint64)


def _vp(a: np.ndarray):
    return a.ctypes.data_as(_dpp)


class DropIn:
    """sgpu_cgsolveq / sgpu_cgsolve on caller-owned storage (Context.dropin):
    q_call() and h_call() solve in place and return Stats; reset() restores the
    initial guesses (the caller's state before the step)."""

    def __init__(self, ctx, qprob, hprob):
        g = ctx.grid
        self.ctx = ctx
        self.q0 = np.array(qprob.q, dtype=np.float64, copy=True)
        self.q = self.q0.copy()
        self.h0 = np.array(hprob.h, dtype=np.float64, copy=True)
        self.h = self.h0.copy()
        self.keep, self.P = ctx._q_ptrs(qprob, self.q)
        self.Dq = np.ascontiguousarray(qprob.D, dtype=np.float64)
        self.ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        self.htmp = np.ascontiguousarray(hprob.htmp, dtype=np.float64)
        self.Dh = np.ascontiguousarray(hprob.D, dtype=np.float64)

    def reset(self):
        np.copyto(self.q, self.q0)
        np.copyto(self.h, self.h0)

    def q_call(self, props) -> "Stats":
        st = Stats()
        pr = props_struct(props)
        P = self.P
        rc = self.ctx.lib.sgpu_cgsolveq(self.ctx.h, self.ctop.ctypes.data_as(_ip), _vp(P["dzz"]), _vp(P["dzf"]),
                                        self.Dq.ctypes.data_as(_dp), _vp(P["q"]), _vp(P["src"]), _vp(P["c"]),
                                        C.byref(pr), C.byref(st))
        self.ctx._check(rc, "sgpu_cgsolveq")
        return st

    def h_call(self, props) -> "Stats":
        st = Stats()
        pr = props_struct(props)
        rc = self.ctx.lib.sgpu_cgsolve(self.ctx.h, self.Dh.ctypes.data_as(_dp), self.h.ctypes.data_as(_dp),
                                       self.htmp.ctypes.data_as(_dp), C.byref(pr), C.byref(st))
        self.ctx._check(rc, "sgpu_cgsolve")
        return st


class SolverError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class Context:
    """One grid resident on one GPU (sgpu_create / sgpu_destroy)."""

    def __init__(self, g: SunGrid, device: int = 0):
        self.lib = load()
        self.grid = g
        self._keep = [g.nfaces, g.neigh, g.face, g.Nk, g.Nke, g.cellp, g.celldist, g.Ac, g.df, g.dg]
        d = GridDesc(g.Nc, g.Ne, g.maxfaces, g.Nkmax,
                     *[a.ctypes.data_as(_ip) for a in self._keep[:7]],
                     *[a.ctypes.data_as(_dp) for a in self._keep[7:]])
        h = C.c_void_p()
        rc = self.lib.sgpu_create(C.byref(d), device, C.byref(h))
        self.h = h
        if rc != OK:
            msg = self.lib.sgpu_last_error(h).decode() if h.value else self.lib.sgpu_status_string(rc).decode()
            if h.value:
                self.lib.sgpu_destroy(h)
            self.h = C.c_void_p()
            raise SolverError(rc, f"sgpu_create: {msg}")
        self.coff = g.coff
        self.eoff = g.eoff

    def close(self):
        if self.h and self.h.value:
            self.lib.sgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self) -> str:
        return self.lib.sgpu_last_error(self.h).decode()

    def _check(self, rc, what, allow=(OK, MAXITER, BREAKDOWN)):
        if rc not in allow:
            raise SolverError(rc, f"{what}: {self.lib.sgpu_status_string(rc).decode()}: {self.error()}")
        return rc

    def set_timeout_ns(self, ns: int):
        self._check(self.lib.sgpu_set_timeout_ns(self.h, int(ns)), "sgpu_set_timeout_ns")

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.lib.sgpu_stream(self.h) or 0)

    def phase_times_ms(self):
        """Device time per phase of the last solve (zero unless built with -DSGPU_PHASE_TIMING)."""
        arr = (C.c_longlong * 8)()
        self.lib.sgpu_phase_times(self.h, arr)
        return [arr[k] / 1e6 for k in range(8)]

    def set_grid(self, ctas: int):
        self._check(self.lib.sgpu_set_grid(self.h, int(ctas)), "sgpu_set_grid")

    # ---- pressure ----
    def _q_ptrs(self, prob, q):
        g = self.grid
        dzz = np.ascontiguousarray(g.dzz)
        dzf = np.ascontiguousarray(g.dzf)
        src = np.ascontiguousarray(prob.src, dtype=np.float64)
        c = np.ascontiguousarray(prob.c, dtype=np.float64)
        keep = [dzz, dzf, src, c, q]
        ptrs = dict(dzz=jagged(dzz, self.coff), dzf=jagged(dzf, self.eoff) if g.Ne else np.zeros(1, np.uint64),
                    src=jagged(src, self.coff), c=jagged(c, self.coff), q=jagged(q, self.coff))
        return keep, ptrs

    def cgsolveq(self, prob, props: SolverProps):
        """The drop-in call: returns (q, Stats) with q a new ragged array."""
        g = self.grid
        q = np.array(prob.q, dtype=np.float64, copy=True)
        keep, P = self._q_ptrs(prob, q)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        st = Stats()
        pr = props_struct(props)
        rc = self.lib.sgpu_cgsolveq(self.h, ctop.ctypes.data_as(_ip), _vp(P["dzz"]), _vp(P["dzf"]),
                                    D.ctypes.data_as(_dp), _vp(P["q"]), _vp(P["src"]), _vp(P["c"]),
                                    C.byref(pr), C.byref(st))
        self._check(rc, "sgpu_cgsolveq")
        return q, st

    def q_upload(self, prob):
        g = self.grid
        q = np.ascontiguousarray(prob.q, dtype=np.float64)
        keep, P = self._q_ptrs(prob, q)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        rc = self.lib.sgpu_q_upload(self.h, ctop.ctypes.data_as(_ip), _vp(P["dzz"]), _vp(P["dzf"]),
                                    D.ctypes.data_as(_dp), _vp(P["q"]), _vp(P["src"]), _vp(P["c"]))
        self._check(rc, "sgpu_q_upload", allow=(OK,))

    def q_solve(self, props: SolverProps) -> Stats:
        st = Stats()
        pr = props_struct(props)
        self._check(self.lib.sgpu_q_solve(self.h, C.byref(pr), C.byref(st)), "sgpu_q_solve")
        return st

    def q_download(self, q0: np.ndarray) -> np.ndarray:
        q = np.array(q0, dtype=np.float64, copy=True)
        ptr = jagged(q, self.coff)
        self._check(self.lib.sgpu_q_download(self.h, _vp(ptr)), "sgpu_q_download", allow=(OK,))
        return q

    # ---- the steps around CGSolveQ ----
    def step_grid(self, st):
        """Uploads the extra gridT fields (normal, grad, computational edges) of step fields st."""
        g = self.grid
        self._step_keep = [np.ascontiguousarray(x, dtype=np.int32) for x in (g.normal, g.grad, st.edgep, st.edgedist)]
        k = self._step_keep
        self._check(self.lib.sgpu_step_grid(self.h, *[x.ctypes.data_as(_ip) for x in k]), "sgpu_step_grid",
                    allow=(OK,))

    def _step_ptrs(self, st):
        g = self.grid
        woff = st.woff
        arrs = {n: np.ascontiguousarray(getattr(st, n), dtype=np.float64) for n in ("u", "utmp2", "w", "wtmp2")}
        P = {"u": jagged(arrs["u"], self.eoff) if g.Ne else np.zeros(1, np.uint64),
             "utmp2": jagged(arrs["utmp2"], self.eoff) if g.Ne else np.zeros(1, np.uint64),
             "w": jagged(arrs["w"], woff), "wtmp2": jagged(arrs["wtmp2"], woff)}
        return arrs, P

    def compute_qsource(self, st, props: SolverProps):
        """ComputeQSource on step fields st: returns (src, D)."""
        g = self.grid
        arrs, P = self._step_ptrs(st)
        dzf = np.ascontiguousarray(g.dzf)
        pdzf = jagged(dzf, self.eoff) if g.Ne else np.zeros(1, np.uint64)
        src = np.zeros(g.n3)
        psrc = jagged(src, self.coff)
        D = np.zeros(max(g.Ne, 1))
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        rc = self.lib.sgpu_compute_qsource(self.h, ctop.ctypes.data_as(_ip), _vp(pdzf), _vp(P["u"]), _vp(P["utmp2"]),
                                           _vp(P["w"]), _vp(P["wtmp2"]), float(props.theta), float(props.dt),
                                           _vp(psrc), D.ctypes.data_as(_dp))
        self._check(rc, "sgpu_compute_qsource", allow=(OK,))
        return src, D[:g.Ne]

    def corrector(self, st, qc, D, props: SolverProps):
        """Corrector with correction qc: returns updated copies (u, w, q) of st's."""
        g = self.grid
        u = np.array(st.u, dtype=np.float64, copy=True)
        w = np.array(st.w, dtype=np.float64, copy=True)
        q = np.array(st.q, dtype=np.float64, copy=True)
        qc = np.ascontiguousarray(qc, dtype=np.float64)
        dzz = np.ascontiguousarray(g.dzz)
        D = np.ascontiguousarray(D, dtype=np.float64)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        etop = np.ascontiguousarray(st.etop, dtype=np.int32)
        pu = jagged(u, self.eoff) if g.Ne else np.zeros(1, np.uint64)
        rc = self.lib.sgpu_corrector(self.h, ctop.ctypes.data_as(_ip), etop.ctypes.data_as(_ip),
                                     _vp(jagged(dzz, self.coff)), _vp(jagged(qc, self.coff)), D.ctypes.data_as(_dp),
                                     float(props.dt), _vp(pu), _vp(jagged(w, st.woff)), _vp(jagged(q, self.coff)))
        self._check(rc, "sgpu_corrector", allow=(OK,))
        return u, w, q

    def pressure_step(self, st, props: SolverProps):
        """ComputeQSource -> CGSolveQ -> Corrector in one call: returns (qc, u, w, q, Stats)."""
        g = self.grid
        u = np.array(st.u, dtype=np.float64, copy=True)
        w = np.array(st.w, dtype=np.float64, copy=True)
        q = np.array(st.q, dtype=np.float64, copy=True)
        qc = np.array(st.qc, dtype=np.float64, copy=True)
        ut2 = np.ascontiguousarray(st.utmp2, dtype=np.float64)
        wt2 = np.ascontiguousarray(st.wtmp2, dtype=np.float64)
        c = np.ascontiguousarray(st.c, dtype=np.float64)
        dzz = np.ascontiguousarray(g.dzz)
        dzf = np.ascontiguousarray(g.dzf)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        etop = np.ascontiguousarray(st.etop, dtype=np.int32)
        E = (lambda a: jagged(a, self.eoff)) if g.Ne else (lambda a: np.zeros(1, np.uint64))
        woff = st.woff
        ptr = [jagged(dzz, self.coff), E(dzf), E(ut2), jagged(wt2, woff), E(u), jagged(w, woff),
               jagged(q, self.coff), jagged(qc, self.coff), jagged(c, self.coff)]
        pr = props_struct(props)
        stt = Stats()
        rc = self.lib.sgpu_pressure_step(self.h, ctop.ctypes.data_as(_ip), etop.ctypes.data_as(_ip),
                                         *[_vp(x) for x in ptr], C.byref(pr), C.byref(stt))
        self._check(rc, "sgpu_pressure_step")
        return qc, u, w, q, stt

    def nonhydrostatic_step(self, st, wf, props: SolverProps):
        """WPredictor -> ComputeQSource -> CGSolveQ -> Corrector in one call, on
        the step's w, q and utmp2 (wf gives the viscosities, histories and
        settings): returns (qc, u, w, q, Cn_W, Cn_W2, Stats)."""
        g = self.grid
        u = np.array(st.u, dtype=np.float64, copy=True)
        w = np.array(st.w, dtype=np.float64, copy=True)
        q = np.array(st.q, dtype=np.float64, copy=True)
        qc = np.array(st.qc, dtype=np.float64, copy=True)
        cw = np.array(wf.Cn_W, dtype=np.float64, copy=True)
        cw2 = np.array(wf.Cn_W2, dtype=np.float64, copy=True)
        ut2 = np.ascontiguousarray(st.utmp2, dtype=np.float64)
        wt2 = np.ascontiguousarray(st.wtmp2, dtype=np.float64)
        c = np.ascontiguousarray(st.c, dtype=np.float64)
        dzz = np.ascontiguousarray(g.dzz)
        dzf = np.ascontiguousarray(g.dzf)
        nt = np.ascontiguousarray(wf.nu_tv, dtype=np.float64)
        nl = np.ascontiguousarray(wf.nu_lax, dtype=np.float64)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        etop = np.ascontiguousarray(st.etop, dtype=np.int32)
        E = (lambda a: jagged(a, self.eoff)) if g.Ne else (lambda a: np.zeros(1, np.uint64))
        woff = st.woff
        f_rows = [jagged(q, self.coff), jagged(nt, self.coff), jagged(nl, self.coff), E(ut2)]
        f = WPredFieldsC(*[_vp(r) for r in f_rows], float(wf.nu), float(wf.nu_H), float(wf.CdW),
                         float(wf.laxWendroff_Vertical), int(wf.nonlinear), int(wf.conserveMomentum), int(wf.n),
                         int(wf.AB))
        ptr = [jagged(dzz, self.coff), E(dzf), E(ut2), jagged(wt2, woff)]
        out = [E(u), jagged(w, woff), jagged(q, self.coff), jagged(qc, self.coff), jagged(c, self.coff),
               jagged(cw, self.coff), jagged(cw2, self.coff)]
        pr = props_struct(props)
        stt = Stats()
        rc = self.lib.sgpu_nonhydrostatic_step(self.h, ctop.ctypes.data_as(_ip), etop.ctypes.data_as(_ip),
                                               *[_vp(x) for x in ptr], C.byref(f), *[_vp(x) for x in out],
                                               C.byref(pr), C.byref(stt))
        self._check(rc, "sgpu_nonhydrostatic_step")
        return qc, u, w, q, cw, cw2, stt

    # ---- the vertical grid of the step ----
    def _vgrid(self, vf):
        g = self.grid
        keep = [np.ascontiguousarray(g.dz, dtype=np.float64), np.ascontiguousarray(g.dv, dtype=np.float64),
                np.ascontiguousarray(vf.dzbot, dtype=np.float64), np.ascontiguousarray(vf.Nkc, dtype=np.int32)]
        v = VGrid(keep[0].ctypes.data_as(_dp), keep[1].ctypes.data_as(_dp), keep[2].ctypes.data_as(_dp),
                  keep[3].ctypes.data_as(_ip), float(vf.smoothbot), float(vf.dzsmall))
        return v, keep

    def update_dz(self, vf, linearFS=0):
        """UpdateDZ (option 0): returns (ctop, etop, dzz, ctopold, etopold, dzzold)."""
        g = self.grid
        v, keep = self._vgrid(vf)
        ctop = np.array(vf.ctop, dtype=np.int32, copy=True)
        etop = np.array(vf.etop, dtype=np.int32, copy=True)
        dzz = np.array(vf.dzz, dtype=np.float64, copy=True)
        ctopold = np.full(g.Nc, -7, dtype=np.int32)
        etopold = np.full(max(g.Ne, 1), -7, dtype=np.int32)
        dzzold = np.full(g.n3, -7.0)
        h = np.ascontiguousarray(vf.h, dtype=np.float64)
        rc = self.lib.sgpu_update_dz(self.h, C.byref(v), h.ctypes.data_as(_dp), int(linearFS), ctop.ctypes.data_as(_ip),
                                     etop.ctypes.data_as(_ip), _vp(jagged(dzz, self.coff)), ctopold.ctypes.data_as(_ip),
                                     etopold.ctypes.data_as(_ip), _vp(jagged(dzzold, self.coff)))
        self._check(rc, "sgpu_update_dz", allow=(OK,))
        return ctop, etop[:g.Ne], dzz, ctopold, etopold[:g.Ne], dzzold

    def set_flux_height(self, vf, dzz=None, etop=None):
        """SetFluxHeight: returns (dzf rows of Nkc levels, dzz after the smoothbot adjustments)."""
        g = self.grid
        v, keep = self._vgrid(vf)
        et = np.ascontiguousarray(vf.etop if etop is None else etop, dtype=np.int32)
        dzz = np.array(vf.dzz if dzz is None else dzz, dtype=np.float64, copy=True)
        dzf = np.full(int(np.sum(vf.Nkc)), -7.0)
        h = np.ascontiguousarray(vf.h, dtype=np.float64)
        uu = np.ascontiguousarray(vf.u, dtype=np.float64)
        rc = self.lib.sgpu_set_flux_height(self.h, C.byref(v), et.ctypes.data_as(_ip), h.ctypes.data_as(_dp),
                                           _vp(jagged(uu, self.eoff)), _vp(jagged(dzz, self.coff)),
                                           _vp(jagged(dzf, vf.foff)))
        self._check(rc, "sgpu_set_flux_height", allow=(OK,))
        return dzf, dzz

    # ---- WPredictor ----
    def wpredictor(self, wf, props: SolverProps, ctop=None, dzz=None):
        """Returns (w, Cn_W, Cn_W2) after one WPredictor on the device."""
        g = self.grid
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (wf.q, wf.nu_tv, wf.nu_lax, wf.utmp2)]
        rows = [jagged(keep[0], self.coff), jagged(keep[1], self.coff), jagged(keep[2], self.coff),
                jagged(keep[3], self.eoff)]
        f = WPredFieldsC(*[_vp(r) for r in rows], float(wf.nu), float(wf.nu_H), float(wf.CdW),
                         float(wf.laxWendroff_Vertical), int(wf.nonlinear), int(wf.conserveMomentum), int(wf.n),
                         int(wf.AB))
        ct = np.ascontiguousarray(g.ctop if ctop is None else ctop, dtype=np.int32)
        zz = np.ascontiguousarray(g.dzz if dzz is None else dzz, dtype=np.float64)
        w = np.array(wf.w, dtype=np.float64, copy=True)
        cw = np.array(wf.Cn_W, dtype=np.float64, copy=True)
        cw2 = np.array(wf.Cn_W2, dtype=np.float64, copy=True)
        pr = props_struct(props)
        rc = self.lib.sgpu_wpredictor(self.h, ct.ctypes.data_as(_ip), _vp(jagged(zz, self.coff)), C.byref(f),
                                      C.byref(pr), _vp(jagged(w, wf.woff)), _vp(jagged(cw, self.coff)),
                                      _vp(jagged(cw2, self.coff)))
        self._check(rc, "sgpu_wpredictor", allow=(OK,))
        return w, cw, cw2

    # ---- UPredictor ----
    def upredictor_grid(self, uf):
        """Edge orderings, marks, normals and every cell's faces (once per grid)."""
        g = self.grid
        ki = [np.ascontiguousarray(a, dtype=np.int32) for a in (uf.bedgep, uf.bedgedist, uf.mark)]
        kd = [np.ascontiguousarray(a, dtype=np.float64) for a in (uf.n1, uf.n2)]
        kf = [np.ascontiguousarray(a, dtype=np.int32) for a in (g.face, g.normal)]
        self._up_keep = ki + kd + kf
        rc = self.lib.sgpu_upredictor_grid(self.h, *[a.ctypes.data_as(_ip) for a in ki],
                                           *[a.ctypes.data_as(_dp) for a in kd], *[a.ctypes.data_as(_ip) for a in kf])
        self._check(rc, "sgpu_upredictor_grid", allow=(OK,))

    def _upred_fields(self, uf):
        g = self.grid
        woff = uf.woff
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (uf.u, uf.w, uf.nu_tv, uf.nu_lax, uf.tau_T,
                                                                      uf.CdT, uf.CdB)]
        rows = [jagged(keep[0], self.eoff), jagged(keep[1], woff), jagged(keep[2], self.coff),
                jagged(keep[3], self.coff)]
        f = UPredFieldsC(*[_vp(r) for r in rows], *[a.ctypes.data_as(_dp) for a in keep[4:]], float(uf.nu),
                         float(uf.laxWendroff_Vertical), float(uf.thetaM), int(uf.nonlinear))
        return f, keep + rows

    def upredictor_vertical(self, uf, props: SolverProps, ctop=None, etop=None, dzz=None, dzf=None):
        """U***, E (computational rows; others 0) and D; returns (utmp, E, D)."""
        g = self.grid
        f, keep = self._upred_fields(uf)
        ct = np.ascontiguousarray(g.ctop if ctop is None else ctop, dtype=np.int32)
        et = np.ascontiguousarray(uf.etop if etop is None else etop, dtype=np.int32)
        zz = np.ascontiguousarray(g.dzz if dzz is None else dzz, dtype=np.float64)
        zf = np.ascontiguousarray(g.dzf if dzf is None else dzf, dtype=np.float64)
        h = np.ascontiguousarray(uf.h, dtype=np.float64)
        utmp = np.array(uf.utmp, dtype=np.float64, copy=True)
        E = np.zeros(max(int(g.Nke.sum()), 1))
        D = np.full(max(g.Ne, 1), -7.0)
        pr = props_struct(props)
        rc = self.lib.sgpu_upredictor_vertical(self.h, ct.ctypes.data_as(_ip), et.ctypes.data_as(_ip),
                                               _vp(jagged(zz, self.coff)), _vp(jagged(zf, self.eoff)),
                                               h.ctypes.data_as(_dp), C.byref(f), C.byref(pr),
                                               _vp(jagged(utmp, self.eoff)), _vp(jagged(E, self.eoff)),
                                               D.ctypes.data_as(_dp))
        self._check(rc, "sgpu_upredictor_vertical", allow=(OK,))
        return utmp, E[:int(g.Nke.sum())], D[:g.Ne]

    def upredictor_rhs(self, uf, props: SolverProps, utmp, h=None, etop=None, dzf=None):
        g = self.grid
        et = np.ascontiguousarray(uf.etop if etop is None else etop, dtype=np.int32)
        zf = np.ascontiguousarray(g.dzf if dzf is None else dzf, dtype=np.float64)
        u = np.ascontiguousarray(uf.u, dtype=np.float64)
        ut = np.ascontiguousarray(utmp, dtype=np.float64)
        hh = np.ascontiguousarray(uf.h if h is None else h, dtype=np.float64)
        htmp = np.zeros(g.Nc)
        pr = props_struct(props)
        rc = self.lib.sgpu_upredictor_rhs(self.h, et.ctypes.data_as(_ip), _vp(jagged(zf, self.eoff)),
                                          _vp(jagged(u, self.eoff)), _vp(jagged(ut, self.eoff)),
                                          hh.ctypes.data_as(_dp), C.byref(pr), htmp.ctypes.data_as(_dp))
        self._check(rc, "sgpu_upredictor_rhs", allow=(OK,))
        return htmp

    def upredictor_finish(self, uf, vf, props: SolverProps, utmp, E, h, ctop, etop, dzz, u=None):
        """Returns (h, active, u, ctop, etop, dzz) after the post-solve steps."""
        g = self.grid
        v, keepv = self._vgrid(vf)
        ct = np.array(ctop, dtype=np.int32, copy=True)
        et = np.array(etop, dtype=np.int32, copy=True)
        zz = np.array(dzz, dtype=np.float64, copy=True)
        ut = np.ascontiguousarray(utmp, dtype=np.float64)
        EE = np.ascontiguousarray(E, dtype=np.float64)
        hh = np.array(h, dtype=np.float64, copy=True)
        active = np.full(g.Nc, 7, dtype=np.uint8)
        uu = np.array(uf.u if u is None else u, dtype=np.float64, copy=True)
        pr = props_struct(props)
        rc = self.lib.sgpu_upredictor_finish(self.h, C.byref(v), C.byref(pr), ct.ctypes.data_as(_ip),
                                             et.ctypes.data_as(_ip), _vp(jagged(zz, self.coff)),
                                             _vp(jagged(ut, self.eoff)), _vp(jagged(EE, self.eoff)),
                                             hh.ctypes.data_as(_dp), active.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                             _vp(jagged(uu, self.eoff)))
        self._check(rc, "sgpu_upredictor_finish", allow=(OK,))
        return hh, active, uu, ct, et, zz

    def upredictor(self, uf, vf, props: SolverProps):
        """The whole UPredictor with CGSolve on the device, from the grid's ctop /
        dzz / dzf and uf.etop; returns a dict like the oracle's."""
        g = self.grid
        v, keepv = self._vgrid(vf)
        f, keep = self._upred_fields(uf)
        ct = np.array(g.ctop, dtype=np.int32, copy=True)
        et = np.array(uf.etop, dtype=np.int32, copy=True)
        zz = np.array(g.dzz, dtype=np.float64, copy=True)
        zf = np.ascontiguousarray(g.dzf, dtype=np.float64)
        u = np.array(uf.u, dtype=np.float64, copy=True)
        h = np.array(uf.h, dtype=np.float64, copy=True)
        utmp = np.array(uf.utmp, dtype=np.float64, copy=True)
        E = np.zeros(max(int(g.Nke.sum()), 1))
        D = np.zeros(max(g.Ne, 1))
        active = np.full(g.Nc, 7, dtype=np.uint8)
        st = Stats()
        pr = props_struct(props)
        rc = self.lib.sgpu_upredictor(self.h, C.byref(v), C.byref(f), C.byref(pr), ct.ctypes.data_as(_ip),
                                      et.ctypes.data_as(_ip), _vp(jagged(zz, self.coff)), _vp(jagged(zf, self.eoff)),
                                      _vp(jagged(u, self.eoff)), h.ctypes.data_as(_dp), _vp(jagged(utmp, self.eoff)),
                                      _vp(jagged(E, self.eoff)), D.ctypes.data_as(_dp),
                                      active.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(st))
        self._check(rc, "sgpu_upredictor")
        return dict(u=u, h=h, utmp=utmp, E=E[:int(g.Nke.sum())], D=D[:g.Ne], ctop=ct, etop=et, dzz=zz,
                    active=active, niters=st.niters, stats=st)

    # ---- free surface ----
    def cgsolve(self, prob, props: SolverProps):
        h = np.array(prob.h, dtype=np.float64, copy=True)
        htmp = np.ascontiguousarray(prob.htmp, dtype=np.float64)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        st = Stats()
        pr = props_struct(props)
        rc = self.lib.sgpu_cgsolve(self.h, D.ctypes.data_as(_dp), h.ctypes.data_as(_dp),
                                   htmp.ctypes.data_as(_dp), C.byref(pr), C.byref(st))
        self._check(rc, "sgpu_cgsolve")
        return h, st

    def dropin(self, qprob, hprob):
        """The two drop-in calls as the reference model makes them: the caller
        owns its rows (here flat copies of the problems' fields, with row
        pointers built once, as phys->qc, grid->dzz ... are), and each call
        solves in place -- q rows (CGSolveQ) and h (CGSolve) overwritten."""
        return DropIn(self, qprob, hprob)

    def h_upload(self, prob):
        h = np.ascontiguousarray(prob.h, dtype=np.float64)
        htmp = np.ascontiguousarray(prob.htmp, dtype=np.float64)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        self._check(self.lib.sgpu_h_upload(self.h, D.ctypes.data_as(_dp), h.ctypes.data_as(_dp),
                                           htmp.ctypes.data_as(_dp)), "sgpu_h_upload", allow=(OK,))

    def h_solve(self, props: SolverProps) -> Stats:
        st = Stats()
        pr = props_struct(props)
        self._check(self.lib.sgpu_h_solve(self.h, C.byref(pr), C.byref(st)), "sgpu_h_solve")
        return st

    def h_download(self, h0: np.ndarray) -> np.ndarray:
        h = np.array(h0, dtype=np.float64, copy=True)
        self._check(self.lib.sgpu_h_download(self.h, h.ctypes.data_as(_dp)), "sgpu_h_download", allow=(OK,))
        return h
