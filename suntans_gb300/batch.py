"""Batched mixed-precision pressure solves (sgpu_batch_* of include/suntans_gb300.h).

    b = Batch(qprecond=1, maxfaces=3, max_slots=..., max_cols=..., max_edge_slots=..., max_instances=256)
    ids = [b.add(problem, tol=1e-10, maxiters=5000) for problem in problems]
    b.run()                       # one persistent launch until every problem is done
    q, stats = b.result(ids[0], problems[0].q)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import GridDesc, OK, SolverError, Stats, _dp, _dpp, _ip, jagged, load


def grid_desc(g):
    keep = [g.nfaces, g.neigh, g.face, g.Nk, g.Nke, g.cellp, g.celldist, g.Ac, g.df, g.dg]
    d = GridDesc(g.Nc, g.Ne, g.maxfaces, g.Nkmax, *[a.ctypes.data_as(_ip) for a in keep[:7]],
                 *[a.ctypes.data_as(_dp) for a in keep[7:]])
    return d, keep


def request_bytes(g, qprecond: int) -> int:
    """Device bytes one problem on grid g occupies in a batch."""
    return int(load().sgpu_batch_bytes_per_request(qprecond, g.maxfaces, g.n3, g.ncomp, int(g.Nke.sum())))


class Batch:
    def __init__(self, qprecond=1, maxfaces=3, max_slots=1 << 20, max_cols=1 << 16, max_edge_slots=1 << 21,
                 max_instances=64, device=0, delta=None, ctas=None):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.sgpu_batch_create(device, qprecond, maxfaces, int(max_slots), int(max_cols),
                                        int(max_edge_slots), int(max_instances), C.byref(h))
        self.h = h
        if rc != OK:
            msg = self.lib.sgpu_batch_last_error(h).decode() if h.value else capi.load().sgpu_status_string(rc).decode()
            if h.value:
                self.lib.sgpu_batch_destroy(h)
            self.h = C.c_void_p()
            raise SolverError(rc, f"sgpu_batch_create: {msg}")
        self.qprecond = qprecond
        self.grids = {}
        if delta is not None or ctas is not None:
            self.set(delta=delta, ctas=ctas)

    def close(self):
        if self.h and self.h.value:
            self.lib.sgpu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        return self.lib.sgpu_batch_last_error(self.h).decode()

    def set(self, delta=None, ctas=None, timeout_ns=None):
        rc = self.lib.sgpu_batch_set(self.h, float(delta or 0.0), -1 if ctas is None else int(ctas),
                                     int(timeout_ns or 0))
        if rc != OK:
            raise SolverError(rc, "sgpu_batch_set")

    def set_fusion(self, form: int):
        """The form of a CG iteration: 1 (default) two passes with the FP32
        solution update run in the next apply pass, 0 two passes with it in
        the update pass (the same bits as 1), 2 one pass per iteration with
        the two reductions merged (qprecond 0/1; qprecond 2 runs it as 1).
        Refused while a problem is in mid-solve under another form."""
        rc = self.lib.sgpu_batch_set_fusion(self.h, int(form))
        if rc != OK:
            raise SolverError(rc, "sgpu_batch_set_fusion")

    def set_stride(self, i: int, stride: int):
        """Problem i advances on every stride-th global iteration of a launch
        (1 = every one); its result bits do not depend on it."""
        rc = self.lib.sgpu_batch_set_stride(self.h, int(i), int(stride))
        if rc != OK:
            raise SolverError(rc, "sgpu_batch_set_stride")

    def set_tile_slots(self, n: int):
        """Storage slots per tile for problems added from now on (4..1024)."""
        rc = self.lib.sgpu_batch_set_tile_slots(self.h, int(n))
        if rc != OK:
            raise SolverError(rc, "sgpu_batch_set_tile_slots")

    def add(self, prob, tol=1e-10, maxiters=5000, resnorm=1.0) -> int:
        """Uploads one pressure problem; returns its id (raises SolverError(OOM) when full)."""
        g = prob.grid
        d, keep = grid_desc(g)
        coff, eoff = g.coff, g.eoff
        dzz = np.ascontiguousarray(g.dzz)
        dzf = np.ascontiguousarray(g.dzf)
        q = np.ascontiguousarray(prob.q, dtype=np.float64)
        src = np.ascontiguousarray(prob.src, dtype=np.float64)
        c = np.ascontiguousarray(prob.c, dtype=np.float64)
        D = np.ascontiguousarray(prob.D, dtype=np.float64)
        ctop = np.ascontiguousarray(g.ctop, dtype=np.int32)
        P = [jagged(dzz, coff), jagged(dzf, eoff) if g.Ne else np.zeros(1, np.uint64), jagged(q, coff),
             jagged(src, coff), jagged(c, coff)]
        idv = C.c_int(-1)
        rc = self.lib.sgpu_batch_add(self.h, C.byref(d), ctop.ctypes.data_as(_ip), P[0].ctypes.data_as(_dpp),
                                     P[1].ctypes.data_as(_dpp), D.ctypes.data_as(_dp), P[2].ctypes.data_as(_dpp),
                                     P[3].ctypes.data_as(_dpp), P[4].ctypes.data_as(_dpp), float(tol), int(maxiters),
                                     float(resnorm), C.byref(idv))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_add: {self.error()}")
        self.grids[idv.value] = g
        return idv.value

    def run(self, max_iters=0):
        """One persistent launch; returns (running, ms, unknown_iterations)."""
        running = C.c_int(0)
        ms = C.c_double(0)
        work = C.c_longlong(0)
        rc = self.lib.sgpu_batch_run(self.h, int(max_iters), C.byref(running), C.byref(ms), C.byref(work))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_run: {self.error()}")
        return running.value, ms.value, work.value

    def launch(self, max_iters=0):
        """Enqueues one launch and returns at once (see `wait`)."""
        rc = self.lib.sgpu_batch_launch(self.h, int(max_iters))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_launch: {self.error()}")

    def wait(self):
        """Waits for the launch in flight; returns (running, ms, unknown_iterations)."""
        running = C.c_int(0)
        ms = C.c_double(0)
        work = C.c_longlong(0)
        rc = self.lib.sgpu_batch_wait(self.h, C.byref(running), C.byref(ms), C.byref(work))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_wait: {self.error()}")
        return running.value, ms.value, work.value

    def state(self, i) -> int:
        return self.lib.sgpu_batch_state(self.h, int(i))

    def result(self, i, q0=None, release=True, out=None):
        """(q, Stats) of a finished problem; q starts from q0 (entries outside the
        active set kept), or the solution is written into `out` (flat ragged
        float64 array of the grid, reused by the caller) when given."""
        g = self.grids[i]
        st = Stats()
        if out is not None:
            q = out
        else:
            if q0 is None:
                q0 = np.zeros(g.n3)
            q = np.array(q0, dtype=np.float64, copy=True)
        ptr = jagged(q, g.coff)
        rc = self.lib.sgpu_batch_result(self.h, int(i), ptr.ctypes.data_as(_dpp), C.byref(st), int(release))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_result: {self.error()}")
        if release:
            self.grids.pop(i, None)
        return q, st

    def release(self, i):
        """Frees problem i's device storage without copying its result."""
        rc = self.lib.sgpu_batch_result(self.h, int(i), None, None, 1)
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_result: {self.error()}")
        self.grids.pop(i, None)

    def resubmit(self, i, src=None, tol=1e-10, maxiters=5000, warm=True):
        """Re-run finished problem i: new right-hand side (None keeps the resident
        one); warm=True starts from its last solution, False from the original guess."""
        g = self.grids[i]
        if src is None:
            p = None
        else:
            src = np.ascontiguousarray(src, dtype=np.float64)
            ptr = jagged(src, g.coff)
            p = ptr.ctypes.data_as(_dpp)
        rc = self.lib.sgpu_batch_resubmit(self.h, int(i), p, float(tol), int(maxiters), int(bool(warm)))
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_resubmit: {self.error()}")

    def stream(self) -> int:
        """The batch's cudaStream_t as an integer handle."""
        return int(self.lib.sgpu_batch_stream(self.h) or 0)

    def use_graph(self, on=True) -> bool:
        return bool(self.lib.sgpu_batch_use_graph(self.h, int(on)))

    def graph_launches(self) -> int:
        return int(self.lib.sgpu_batch_graph_launches(self.h))

    def phase_times_ms(self):
        """Per-phase device time of the last launch (zero unless built with -DSGPU_PHASE_TIMING)."""
        arr = (C.c_longlong * 8)()
        self.lib.sgpu_batch_phase_times(self.h, arr)
        names = ["owner_fin_apply", "apply", "update", "merge64", "residual64", "setup1", "setup2", "setup3"]
        return {n: arr[k] / 1e6 for k, n in enumerate(names)}

    def stats(self, i):
        st = Stats()
        rc = self.lib.sgpu_batch_result(self.h, int(i), None, C.byref(st), 0)
        if rc != OK:
            raise SolverError(rc, f"sgpu_batch_result: {self.error()}")
        return st


def capacity_for(grids, qprecond=1, slack=1.0):
    """Arena sizes (slots, cols, edge slots, instances) that hold all `grids` at once."""
    slots = sum(g.n3 for g in grids)
    cols = sum(g.ncomp for g in grids)
    eslots = sum(int(g.Nke.sum()) for g in grids)
    return dict(max_slots=int(slots * slack) + 16, max_cols=int(cols * slack) + 16,
                max_edge_slots=int(eslots * slack) + 16, max_instances=len(grids))
