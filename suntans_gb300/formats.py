"""The reference's grid and field files, read and written on the host.

A SUNTANS run reads its grid from the files that the grid step (``sun -g``)
leaves for each processor P (ReadGrid, main/gridio.c:54-187):

``celldata.dat.P``  one line per cell (ReadCellCenteredData gridio.c:631-661,
                    WriteCellCenteredData 664-685):
                    ``nfaces xv yv Ac dv Nk face[nf] neigh[nf] normal[nf] def[nf] cells[nf] mnptr``
``edgedata.dat.P``  one line per edge (gridio.c:687-725):
                    ``df dg n1 n2 xe ye Nke Nkc grad0 grad1 gradf0 gradf1 mark node0 node1 edge_id eptr``
``nodes.dat.P``     one line per node (ReadNodalData gridio.c:728-783, WriteNodalData 785-830)
``topology.dat.P``  neighbour processors and the cell / edge orderings
                    (gridio.c:365-477): celldist, edgedist, cellp, edgep
``vertspace.dat``   the Nkmax layer thicknesses (gridio.c:496-512)
``cells.dat.P``, ``edges.dat.P``  the plan-view triangulation (WriteCellsData /
                    WriteEdgesData gridio.c:558-629, with nfaces and edge_id).

The grid step itself starts from the input triangulation (ReadMainGrid,
gridio.c:256-266), read by `read_main_grid`:

``points.dat``      ``x y mark`` per node (ReadPointsData gridio.c:515-525)
``edges.dat``       ``n1 n2 mark grad0 grad1 [edge_id]`` per edge (ReadEdgesData
                    gridio.c:535-556; edge_id only when the first line has more
                    than 5 columns)
``cells.dat``       ``[nfaces] xv yv node[nfaces] neigh[nfaces]`` per cell
                    (ReadCellsData gridio.c:574-611; nfaces only when the first
                    line has more than 8 columns, else every cell has 3 faces)

Columns are counted on the first line as getNumColumns does
(fileio.c:205-228): a blank or tab after a character that is not a blank, a
tab or the start of the file starts a column, and a blank right before the
first newline takes one back.

Every reader follows the reference's tokenizer (getfield, main/fileio.c:137-174):
fields are separated by blanks, tabs, newlines or carriage returns; a field with
a character other than ``0-9 . + - e`` is skipped; the value is the longest
number at the start of the field (strtod), 0 when there is none; integer fields
are that value truncated toward zero.  Line counts (getsize, fileio.c:183-196)
give the number of cells, edges and nodes.  One difference: where the reference
would read past the end of a short file as zeros, these readers raise.

Field output (main/physio.c:29-105) and the restart file (StoreFile, written at
physio.c:343-393, read back at 407-483) are raw native-endian doubles in the
layouts of `write_2d`, `write_3d` and `write_store` / `read_store`.

Writers use the reference's printf formats, so a grid built here (see
`GridFiles.from_sungrid`) is read by the reference exactly as by `read_grid`.
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import Dict, List, Optional, Sequence

import numpy as np

from .grid import SunGrid

I32 = np.int32
F64 = np.float64

MAXBCTYPES = 4        # main/grid.h:24 -> celldist has MAXBCTYPES-1 entries
MAXMARKS = 7          # main/grid.h:25 -> edgedist has MAXMARKS-1 entries
EMPTY = 999999.0      # main/suntans.h:28, written below a column's bottom

DEFAULT_NAMES = {     # the keys of suntans.dat (examples/*/rundata/suntans.dat)
    "celldata": "celldata.dat", "edgedata": "edgedata.dat", "nodes": "nodes.dat",
    "topology": "topology.dat", "vertspace": "vertspace.dat", "cells": "cells.dat",
    "edges": "edges.dat", "points": "points.dat",
}

_SEP = re.compile(rb"[ \t\n\r]+")
_BAD = re.compile(rb"[^0-9.+\-e \t\n\r]")
_FIELD_OK = re.compile(rb"[0-9.+\-e]+")
_PREFIX = re.compile(rb"[+-]?(?:[0-9]+\.?[0-9]*|\.[0-9]+)(?:e[+-]?[0-9]+)?")


def _strtod_prefix(tok: bytes) -> float:
    m = _PREFIX.match(tok)
    return float(m.group()) if m else 0.0


def read_fields(path: str) -> np.ndarray:
    """All numeric fields of a file as doubles, in the order getfield returns them."""
    with open(path, "rb") as f:
        data = f.read()
    toks = [t for t in _SEP.split(data) if t]
    if not toks:
        return np.zeros(0, dtype=F64)
    if _BAD.search(data) is None:
        try:
            return np.asarray(toks).astype(F64)
        except ValueError:
            pass
    return np.array([_strtod_prefix(t) for t in toks if _FIELD_OK.fullmatch(t)], dtype=F64)


def count_lines(path: str) -> int:
    """Number of newline characters (getsize, main/fileio.c:183-196)."""
    with open(path, "rb") as f:
        return f.read().count(b"\n")


def _trunc(x: np.ndarray) -> np.ndarray:
    return np.trunc(x).astype(I32)


class _Fields:
    def __init__(self, vals: np.ndarray, path: str):
        self.v, self.p, self.path = vals, 0, path

    def take(self, n: int) -> np.ndarray:
        if self.p + n > self.v.size:
            raise ValueError(f"{self.path}: file ends after {self.v.size} fields")
        out = self.v[self.p:self.p + n]
        self.p += n
        return out

    def one(self) -> float:
        return float(self.take(1)[0])


def _jagged(counts: np.ndarray) -> np.ndarray:
    o = np.zeros(counts.size + 1, dtype=np.int64)
    np.cumsum(counts, out=o[1:])
    return o


@dataclasses.dataclass
class GridFiles:
    """One processor's run-time grid: every array ReadGrid fills (gridT, main/grid.h:32-149).

    Per-face arrays are ``[Nc*maxfaces]`` with unused slots ``-1`` (ints) or 0.
    The nodal neighbour lists are stored flat with offset arrays."""
    maxfaces: int
    Nkmax: int
    # celldata
    nfaces: np.ndarray
    xv: np.ndarray
    yv: np.ndarray
    Ac: np.ndarray
    dv: np.ndarray
    Nk: np.ndarray
    face: np.ndarray
    neigh: np.ndarray
    normal: np.ndarray
    def_: np.ndarray
    cells: np.ndarray
    mnptr: np.ndarray
    # edgedata
    df: np.ndarray
    dg: np.ndarray
    n1: np.ndarray
    n2: np.ndarray
    xe: np.ndarray
    ye: np.ndarray
    Nke: np.ndarray
    Nkc: np.ndarray
    grad: np.ndarray       # [2*Ne]
    gradf: np.ndarray      # [2*Ne]
    mark: np.ndarray
    edges: np.ndarray      # [2*Ne] node ids
    edge_id: np.ndarray
    eptr: np.ndarray
    # topology
    numprocs: int
    myneighs: np.ndarray
    cell_send: List[np.ndarray]
    cell_recv: List[np.ndarray]
    edge_send: List[np.ndarray]
    edge_recv: List[np.ndarray]
    celldist: np.ndarray   # [MAXBCTYPES-1]
    edgedist: np.ndarray   # [MAXMARKS-1]
    cellp: np.ndarray
    edgep: np.ndarray
    # nodes
    node_id: np.ndarray
    xp: np.ndarray
    yp: np.ndarray
    ppneighs: np.ndarray
    ppoff: np.ndarray
    peneighs: np.ndarray
    peoff: np.ndarray
    pcneighs: np.ndarray
    pcoff: np.ndarray
    Actotal: np.ndarray
    Nkp: np.ndarray
    # vertspace
    dz: np.ndarray

    @property
    def Nc(self) -> int:
        return int(self.nfaces.size)

    @property
    def Ne(self) -> int:
        return int(self.df.size)

    @property
    def Np(self) -> int:
        return int(self.xp.size)

    # ------------------------------------------------------------------
    def to_sungrid(self, name: str = "grid") -> SunGrid:
        """The solver's view of this grid, in the state the reference holds right
        after reading it: ctop = 0 (gridio.c:182-186) and dzz = dz on every level
        (InitializeVerticalGrid, main/phys.c:795-801).  dzf starts as dzz on the
        edge's Nke levels, the smaller of the two cells' thicknesses at the bottom
        face and the larger above (SetFluxHeight with u = 0).  UpdateDZ and
        SetFluxHeight bring both to the free surface (`Context.update_dz`,
        `Context.set_flux_height`)."""
        Nc, Ne = self.Nc, self.Ne
        coff = _jagged(self.Nk)
        cell = np.repeat(np.arange(Nc), self.Nk)
        k = np.arange(int(coff[-1])) - coff[cell]
        dzz = self.dz[k].astype(F64)
        eoff = _jagged(self.Nke)
        edge = np.repeat(np.arange(Ne), self.Nke)
        ke = np.arange(int(eoff[-1])) - eoff[edge]
        dzf = self.dz[ke].astype(F64)
        return SunGrid(Nc=Nc, Ne=Ne, maxfaces=self.maxfaces, Nkmax=self.Nkmax, nfaces=self.nfaces,
                       neigh=self.neigh, face=self.face, Nk=self.Nk, Nke=self.Nke,
                       ctop=np.zeros(Nc, dtype=I32), cellp=self.cellp, celldist=self.celldist[:3],
                       Ac=self.Ac, df=self.df, dg=self.dg, dzz=dzz, dzf=dzf, normal=self.normal,
                       grad=self.grad, xv=self.xv, yv=self.yv, dz=self.dz, dv=self.dv,
                       xp=self.xp, yp=self.yp, cnodes=self.cells, enodes=self.edges, mark=self.mark,
                       name=name)

    def computational_edges(self) -> np.ndarray:
        """edgep[edgedist[0]:edgedist[1]]: edges of mark 0 or 5 (main/grid.c:1666-1672)."""
        return self.edgep[self.edgedist[0]:self.edgedist[1]]

    # ------------------------------------------------------------------
    @classmethod
    def from_sungrid(cls, g: SunGrid) -> "GridFiles":
        """Grid files for a grid built by `gridgen` (plan-view geometry required).

        Derived entries follow the reference's definitions: ``normal`` +1 where
        the cell is grad[0]; ``n1, n2`` the unit normal from grad[0] towards
        grad[1]; ``def`` the distance from the Voronoi point to the face;
        ``xe, ye`` the face midpoint; ``Nkc`` the deeper cell's Nk; ``gradf``
        each cell's face slot of the edge; cells ordered computational first
        (mark-3 cells after, main/grid.c:1652-1664) and edges by mark
        (1666-1679); one processor, so ``mnptr`` and ``eptr`` are the
        identity and the topology has no neighbours."""
        if g.xp is None or g.cnodes is None or g.enodes is None or g.mark is None:
            raise ValueError("grid has no plan-view geometry (xp, cnodes, enodes, mark)")
        Nc, Ne, mf = g.Nc, g.Ne, g.maxfaces
        from .gridgen import edge_normals, edges_by_mark
        grad = g.grad.reshape(Ne, 2)
        en = g.enodes.reshape(Ne, 2)
        x0, y0 = g.xp[en[:, 0]], g.yp[en[:, 0]]
        x1, y1 = g.xp[en[:, 1]], g.yp[en[:, 1]]
        c0 = grad[:, 0]
        nx, ny = edge_normals(g)
        slot = np.arange(mf)[None, :] < g.nfaces[:, None]
        fe = np.where(slot, g.face.reshape(Nc, mf), 0)
        cellof = np.repeat(np.arange(Nc), mf).reshape(Nc, mf)
        def_ = np.abs((g.xv[cellof] - x0[fe]) * nx[fe] + (g.yv[cellof] - y0[fe]) * ny[fe])
        def_ = np.where(slot, def_, 0.0).ravel()
        gradf = -np.ones((Ne, 2), dtype=I32)
        for s in range(mf):
            cs = np.nonzero(g.nfaces > s)[0]
            e = g.face[cs * mf + s]
            side = np.where(grad[e, 0] == cs, 0, 1)
            gradf[e, side] = s
        interior = grad[:, 1] >= 0
        Nkc = np.where(interior, np.maximum(g.Nk[c0], g.Nk[np.maximum(grad[:, 1], 0)]), g.Nk[c0]).astype(I32)
        mark = g.mark.astype(I32)
        edgep, edgedist = edges_by_mark(mark)
        # nodal neighbours (points, edges, cells around each node)
        Np = g.xp.size
        pp_a = np.concatenate([en[:, 0], en[:, 1]])
        pp_b = np.concatenate([en[:, 1], en[:, 0]])
        ppneighs, ppoff = _group(pp_a, pp_b, Np)
        peneighs, peoff = _group(pp_a, np.concatenate([np.arange(Ne), np.arange(Ne)]), Np)
        cn = g.cnodes.reshape(Nc, mf)
        pc_a = cn[slot]
        pc_b = cellof[slot]
        pcneighs, pcoff = _group(pc_a, pc_b, Np)
        zi = np.zeros(0, dtype=I32)
        return cls(maxfaces=mf, Nkmax=g.Nkmax, nfaces=g.nfaces.copy(), xv=g.xv.astype(F64),
                   yv=g.yv.astype(F64), Ac=g.Ac.copy(), dv=np.asarray(g.dv, dtype=F64), Nk=g.Nk.copy(),
                   face=np.where(slot.ravel(), g.face, -1).astype(I32),
                   neigh=np.where(slot.ravel(), g.neigh, -1).astype(I32),
                   normal=np.where(slot.ravel(), g.normal, 0).astype(I32), def_=def_,
                   cells=np.where(slot.ravel(), g.cnodes, -1).astype(I32), mnptr=np.arange(Nc, dtype=I32),
                   df=g.df.copy(), dg=g.dg.copy(), n1=nx, n2=ny, xe=0.5 * (x0 + x1), ye=0.5 * (y0 + y1),
                   Nke=g.Nke.copy(), Nkc=Nkc, grad=g.grad.astype(I32).copy(), gradf=gradf.ravel(), mark=mark,
                   edges=g.enodes.astype(I32).copy(), edge_id=np.zeros(Ne, dtype=I32),
                   eptr=np.arange(Ne, dtype=I32), numprocs=1, myneighs=zi, cell_send=[], cell_recv=[],
                   edge_send=[], edge_recv=[],
                   celldist=np.concatenate([g.celldist[:3]]).astype(I32), edgedist=edgedist,
                   cellp=g.cellp.copy(), edgep=edgep, node_id=np.arange(Np, dtype=I32), xp=g.xp.astype(F64),
                   yp=g.yp.astype(F64), ppneighs=ppneighs, ppoff=ppoff, peneighs=peneighs, peoff=peoff,
                   pcneighs=pcneighs, pcoff=pcoff, Actotal=np.zeros(0, dtype=F64),
                   Nkp=np.zeros(Np, dtype=I32), dz=np.asarray(g.dz, dtype=F64))


def _group(keys: np.ndarray, vals: np.ndarray, n: int):
    """Values grouped by key (0..n-1), each group sorted, as a flat list + offsets."""
    order = np.lexsort((vals, keys))
    k, v = keys[order], vals[order]
    counts = np.bincount(k, minlength=n)
    return v.astype(I32), _jagged(counts)


# ----------------------------------------------------------------------------
# reading
# ----------------------------------------------------------------------------
def _names(names: Optional[Dict[str, str]]) -> Dict[str, str]:
    out = dict(DEFAULT_NAMES)
    if names:
        out.update(names)
    return out


def read_grid(datadir: str, proc: int = 0, maxfaces: int = 3, Nkmax: Optional[int] = None,
              names: Optional[Dict[str, str]] = None) -> GridFiles:
    """Read one processor's run-time grid the way ReadGrid does (main/gridio.c:54-187).

    ``maxfaces`` and ``Nkmax`` are the suntans.dat values (maxFaces, Nkmax);
    ``Nkmax`` defaults to the length of vertspace.dat."""
    nm = _names(names)
    P = lambda key: os.path.join(datadir, f"{nm[key]}.{proc}")
    cpath, epath, npath, tpath = P("celldata"), P("edgedata"), P("nodes"), P("topology")
    vpath = os.path.join(datadir, nm["vertspace"])
    Nc, Ne, Np = count_lines(cpath), count_lines(epath), count_lines(npath)

    # topology (ReadTopologyData gridio.c:365-423)
    t = _Fields(read_fields(tpath), tpath)
    numprocs = int(t.one())
    nneigh = int(t.one())
    myneighs = _trunc(t.take(nneigh))
    cs, cr, es, er = [], [], [], []
    for _ in range(nneigh):
        n_cs, n_cr, n_es, n_er = (int(x) for x in t.take(4))
        cs.append(_trunc(t.take(n_cs)))
        cr.append(_trunc(t.take(n_cr)))
        es.append(_trunc(t.take(n_es)))
        er.append(_trunc(t.take(n_er)))
    celldist = _trunc(t.take(MAXBCTYPES - 1))
    edgedist = _trunc(t.take(MAXMARKS - 1))
    cellp = _trunc(t.take(Nc))
    edgep = _trunc(t.take(Ne))

    # celldata (ReadCellCenteredData gridio.c:631-661)
    cv = read_fields(cpath)
    mf = int(maxfaces)
    start = np.zeros(Nc + 1, dtype=np.int64)
    nfa = np.zeros(Nc, dtype=I32)
    p = 0
    for i in range(Nc):
        if p >= cv.size:
            raise ValueError(f"{cpath}: file ends after {cv.size} fields")
        nf = int(cv[p])
        if nf > mf:
            raise ValueError(f"{cpath}: cell {i} has {nf} faces, more than maxFaces {mf}")
        nfa[i] = nf
        start[i] = p
        p += 7 + 5 * max(nf, 0)
    start[Nc] = p
    if p > cv.size:
        raise ValueError(f"{cpath}: file ends after {cv.size} fields")
    s = start[:Nc]
    xv, yv, Ac, dv = cv[s + 1], cv[s + 2], cv[s + 3], cv[s + 4]
    Nk = _trunc(cv[s + 5])
    face = -np.ones((Nc, mf), dtype=I32)
    neigh = -np.ones((Nc, mf), dtype=I32)
    normal = np.zeros((Nc, mf), dtype=I32)
    def_ = np.zeros((Nc, mf), dtype=F64)
    cells = -np.ones((Nc, mf), dtype=I32)
    nf64 = nfa.astype(np.int64)
    for f in range(mf):
        m = nfa > f
        b = s[m] + 6 + f
        n = nf64[m]
        face[m, f] = _trunc(cv[b])
        neigh[m, f] = _trunc(cv[b + n])
        normal[m, f] = _trunc(cv[b + 2 * n])
        def_[m, f] = cv[b + 3 * n]
        cells[m, f] = _trunc(cv[b + 4 * n])
    mnptr = _trunc(cv[s + 6 + 5 * nf64])

    # edgedata (ReadEdgeCenteredData gridio.c:687-712), 17 fields per edge
    ev = read_fields(epath)
    if ev.size < 17 * Ne:
        raise ValueError(f"{epath}: file ends after {ev.size} fields")
    E = ev[:17 * Ne].reshape(Ne, 17)

    # nodes (ReadNodalData gridio.c:728-783)
    nv = _Fields(read_fields(npath), npath)
    node_id = np.zeros(Np, dtype=I32)
    xp = np.zeros(Np, dtype=F64)
    yp = np.zeros(Np, dtype=F64)
    lists = {k: [] for k in ("pp", "pe", "pc", "ac")}
    counts = {k: np.zeros(Np, dtype=np.int64) for k in lists}
    for n in range(Np):
        node_id[n] = int(nv.one())
        xp[n] = nv.one()
        yp[n] = nv.one()
        for key, conv in (("pp", _trunc), ("pe", _trunc), ("pc", _trunc), ("ac", None)):
            c = int(nv.one())
            vals = nv.take(c)
            counts[key][n] = c
            lists[key].append(conv(vals) if conv else vals.copy())
    cat = lambda key, dt: (np.concatenate(lists[key]).astype(dt) if Np else np.zeros(0, dtype=dt))

    # vertspace (ReadVertSpaceData gridio.c:496-503)
    vv = read_fields(vpath)
    nk = int(Nkmax) if Nkmax is not None else count_lines(vpath)
    if vv.size < nk:
        raise ValueError(f"{vpath}: {vv.size} values for Nkmax {nk}")

    return GridFiles(maxfaces=mf, Nkmax=nk, nfaces=nfa, xv=xv, yv=yv, Ac=Ac, dv=dv, Nk=Nk,
                     face=face.ravel(), neigh=neigh.ravel(), normal=normal.ravel(), def_=def_.ravel(),
                     cells=cells.ravel(), mnptr=mnptr,
                     df=E[:, 0].copy(), dg=E[:, 1].copy(), n1=E[:, 2].copy(), n2=E[:, 3].copy(),
                     xe=E[:, 4].copy(), ye=E[:, 5].copy(), Nke=_trunc(E[:, 6]), Nkc=_trunc(E[:, 7]),
                     grad=_trunc(E[:, 8:10]).ravel(), gradf=_trunc(E[:, 10:12]).ravel(),
                     mark=_trunc(E[:, 12]), edges=_trunc(E[:, 13:15]).ravel(), edge_id=_trunc(E[:, 15]),
                     eptr=_trunc(E[:, 16]), numprocs=numprocs, myneighs=myneighs, cell_send=cs,
                     cell_recv=cr, edge_send=es, edge_recv=er, celldist=celldist, edgedist=edgedist,
                     cellp=cellp, edgep=edgep, node_id=node_id, xp=xp, yp=yp,
                     ppneighs=cat("pp", I32), ppoff=_jagged(counts["pp"]),
                     peneighs=cat("pe", I32), peoff=_jagged(counts["pe"]),
                     pcneighs=cat("pc", I32), pcoff=_jagged(counts["pc"]),
                     Actotal=cat("ac", F64), Nkp=counts["ac"].astype(I32), dz=vv[:nk].copy())


# ----------------------------------------------------------------------------
# writing (the reference's printf formats)
# ----------------------------------------------------------------------------
def _e(x) -> str:
    return "%e" % x


def write_grid(gf: GridFiles, datadir: str, proc: int = 0, names: Optional[Dict[str, str]] = None) -> None:
    """Write the files ReadGrid reads, as the reference's grid step writes them
    (OutputGridData, main/gridio.c:275-327): celldata, edgedata, nodes,
    topology, cells and edges for processor ``proc``, and vertspace.dat."""
    nm = _names(names)
    os.makedirs(datadir, exist_ok=True)
    P = lambda key: os.path.join(datadir, f"{nm[key]}.{proc}")
    mf = gf.maxfaces
    Nc, Ne, Np = gf.Nc, gf.Ne, gf.Np

    with open(P("celldata"), "w") as f:     # WriteCellCenteredData gridio.c:664-685
        for i in range(Nc):
            nf = int(gf.nfaces[i])
            b = i * mf
            parts = ["%d %e %e %e %e %d " % (nf, gf.xv[i], gf.yv[i], gf.Ac[i], gf.dv[i], gf.Nk[i])]
            parts += ["%d " % v for v in gf.face[b:b + nf]]
            parts += ["%d " % v for v in gf.neigh[b:b + nf]]
            parts += ["%d " % v for v in gf.normal[b:b + nf]]
            parts += ["%e " % v for v in gf.def_[b:b + nf]]
            parts += ["%d " % v for v in gf.cells[b:b + nf]]
            parts.append("%d \n" % gf.mnptr[i])
            f.write("".join(parts))

    with open(P("edgedata"), "w") as f:     # WriteEdgeCenteredData gridio.c:714-725
        g2 = gf.grad.reshape(Ne, 2)
        gf2 = gf.gradf.reshape(Ne, 2)
        e2 = gf.edges.reshape(Ne, 2)
        for j in range(Ne):
            f.write("%e %e %e %e %e %e %d %d %d %d %d %d %d %d %d %d %d\n" % (
                gf.df[j], gf.dg[j], gf.n1[j], gf.n2[j], gf.xe[j], gf.ye[j], gf.Nke[j], gf.Nkc[j],
                g2[j, 0], g2[j, 1], gf2[j, 0], gf2[j, 1], gf.mark[j], e2[j, 0], e2[j, 1],
                gf.edge_id[j], gf.eptr[j]))

    ac_off = _jagged(gf.Nkp.astype(np.int64))
    with open(P("nodes"), "w") as f:        # WriteNodalData gridio.c:785-830
        for n in range(Np):
            parts = ["%d %e %e " % (gf.node_id[n], gf.xp[n], gf.yp[n])]
            for lst, off in ((gf.ppneighs, gf.ppoff), (gf.peneighs, gf.peoff), (gf.pcneighs, gf.pcoff)):
                a, b = int(off[n]), int(off[n + 1])
                parts.append("%d " % (b - a))
                parts += ["%d " % v for v in lst[a:b]]
            a, b = int(ac_off[n]), int(ac_off[n + 1])
            parts.append("%d " % gf.Nkp[n])
            parts += ["%e " % v for v in gf.Actotal[a:b]]
            parts.append("\n")
            f.write("".join(parts))

    with open(P("topology"), "w") as f:     # WriteTopologyData gridio.c:431-477
        f.write("%d %d\n" % (gf.numprocs, gf.myneighs.size))
        f.write("".join("%d " % v for v in gf.myneighs) + "\n")
        for q in range(gf.myneighs.size):
            f.write("%d %d %d %d\n" % (gf.cell_send[q].size, gf.cell_recv[q].size,
                                       gf.edge_send[q].size, gf.edge_recv[q].size))
            for lst in (gf.cell_send[q], gf.cell_recv[q], gf.edge_send[q], gf.edge_recv[q]):
                f.write("".join("%d " % v for v in lst) + "\n")
        for arr in (gf.celldist, gf.edgedist, gf.cellp, gf.edgep):
            f.write("".join("%d " % v for v in arr) + "\n")

    with open(P("cells"), "w") as f:        # WriteCellsData gridio.c:614-629, "with nfaces"
        for i in range(Nc):
            nf = int(gf.nfaces[i])
            b = i * mf
            f.write("%d " % nf + "%e %e " % (gf.xv[i], gf.yv[i])
                    + "".join("%d " % v for v in gf.cells[b:b + nf])
                    + "".join("%d " % v for v in gf.neigh[b:b + nf]) + "\n")

    with open(P("edges"), "w") as f:        # WriteEdgesData gridio.c:558-573, "with edge_id"
        g2 = gf.grad.reshape(Ne, 2)
        e2 = gf.edges.reshape(Ne, 2)
        for j in range(Ne):
            f.write("%d %d %d %d %d %d \n" % (e2[j, 0], e2[j, 1], gf.mark[j], g2[j, 0], g2[j, 1], gf.edge_id[j]))

    with open(os.path.join(datadir, nm["vertspace"]), "w") as f:   # WriteVertSpaceData gridio.c:506-512
        f.write("".join("%e\n" % v for v in gf.dz))


# ----------------------------------------------------------------------------
# the input triangulation (points, edges, cells)
# ----------------------------------------------------------------------------
COLUMNS_IN_TRIANGLE_CELLS_FILE = 8   # cells.dat columns without nfaces (gridio.c:16)
COLUMNS_IN_TRIANGLE_EDGES_FILE = 5   # edges.dat columns without edge_id (gridio.c:17)
DEFAULT_NFACES = 3                   # main/suntans.h:33


def get_num_columns(path: str) -> int:
    """Columns of a file's first line, counted as getNumColumns counts them
    (main/fileio.c:205-228)."""
    with open(path, "rb") as f:
        data = f.read()
    n, old = 1, 0
    for ch in data:
        if ch in (0x20, 0x09) and old not in (0x20, 0x09, 0):
            n += 1
        if ch == 0x0A:
            if old == 0x20:
                n -= 1
            break
        old = ch
    return n


@dataclasses.dataclass
class MainGrid:
    """The input triangulation that ReadMainGrid fills (gridT.xp, yp, edges,
    mark, grad, edge_id, nfaces, xv, yv, cells, neigh).  cells and neigh are
    [Nc, maxfaces] with -1 past a cell's nfaces."""
    maxfaces: int
    xp: np.ndarray
    yp: np.ndarray
    edges: np.ndarray      # [Ne, 2] node indices
    mark: np.ndarray
    grad: np.ndarray       # [Ne, 2] cell indices (-1 outside)
    edge_id: np.ndarray
    nfaces: np.ndarray
    xv: np.ndarray
    yv: np.ndarray
    cells: np.ndarray      # [Nc, maxfaces] node indices
    neigh: np.ndarray      # [Nc, maxfaces] neighbour cells (-1: none)

    @property
    def Np(self) -> int:
        return int(self.xp.size)

    @property
    def Ne(self) -> int:
        return int(self.mark.size)

    @property
    def Nc(self) -> int:
        return int(self.nfaces.size)


def read_points(path: str):
    """(xp, yp) of every node line (ReadPointsData, gridio.c:515-525: the third
    field, the node's marker, is read and dropped)."""
    Np = count_lines(path)
    v = _Fields(read_fields(path), path).take(3 * Np).reshape(Np, 3)
    return v[:, 0].copy(), v[:, 1].copy()


def read_edges(path: str):
    """(edges [Ne, 2], mark, grad [Ne, 2], edge_id) as ReadEdgesData reads
    them (gridio.c:535-556); edge_id is 0 where the file has no such column."""
    Ne = count_lines(path)
    ncol = 6 if get_num_columns(path) > COLUMNS_IN_TRIANGLE_EDGES_FILE else 5
    v = _trunc(_Fields(read_fields(path), path).take(ncol * Ne)).reshape(Ne, ncol)
    edge_id = v[:, 5].copy() if ncol == 6 else np.zeros(Ne, dtype=I32)
    return v[:, 0:2].copy(), v[:, 2].copy(), v[:, 3:5].copy(), edge_id


def read_cells(path: str, maxfaces: int):
    """(nfaces, xv, yv, cells [Nc, maxfaces], neigh [Nc, maxfaces]) as
    ReadCellsData reads them (gridio.c:574-611).  A cell with more faces than
    maxfaces raises, where the reference stops with an error."""
    Nc = count_lines(path)
    with_nf = get_num_columns(path) > COLUMNS_IN_TRIANGLE_CELLS_FILE
    fl = _Fields(read_fields(path), path)
    nfaces = np.full(Nc, DEFAULT_NFACES, dtype=I32)
    xv = np.zeros(Nc, dtype=F64)
    yv = np.zeros(Nc, dtype=F64)
    cells = -np.ones((Nc, maxfaces), dtype=I32)
    neigh = -np.ones((Nc, maxfaces), dtype=I32)
    for n in range(Nc):
        if with_nf:
            nf = int(np.trunc(fl.one()))
            if nf > maxfaces:
                raise ValueError(f"{path}: cell {n} has {nf} faces, more than maxFaces {maxfaces}")
            nfaces[n] = nf
        nf = int(nfaces[n])
        xv[n] = fl.one()
        yv[n] = fl.one()
        if nf > 0:
            cells[n, :nf] = _trunc(fl.take(nf))
            neigh[n, :nf] = _trunc(fl.take(nf))
    return nfaces, xv, yv, cells, neigh


def read_main_grid(datadir: str, maxfaces: int = DEFAULT_NFACES,
                   names: Optional[Dict[str, str]] = None) -> MainGrid:
    """Read the input triangulation the way ReadMainGrid does (gridio.c:256-266):
    points, edges and cells files of ``datadir`` (names as in suntans.dat)."""
    nm = _names(names)
    xp, yp = read_points(os.path.join(datadir, nm["points"]))
    edges, mark, grad, edge_id = read_edges(os.path.join(datadir, nm["edges"]))
    nfaces, xv, yv, cells, neigh = read_cells(os.path.join(datadir, nm["cells"]), maxfaces)
    return MainGrid(maxfaces=maxfaces, xp=xp, yp=yp, edges=edges, mark=mark, grad=grad, edge_id=edge_id,
                    nfaces=nfaces, xv=xv, yv=yv, cells=cells, neigh=neigh)


def write_main_grid(mg: MainGrid, datadir: str, names: Optional[Dict[str, str]] = None, with_nfaces: bool = True,
                    with_edge_id: bool = True) -> None:
    """Write the input triangulation in the reference's formats:
    WritePointsData (gridio.c:527-533, marker written as 0), WriteEdgesData
    (558-572) and WriteCellsData (613-629), with or without the nfaces and
    edge_id columns."""
    nm = _names(names)
    os.makedirs(datadir, exist_ok=True)
    with open(os.path.join(datadir, nm["points"]), "w") as f:
        f.write("".join("%e %e 0\n" % (x, y) for x, y in zip(mg.xp, mg.yp)))
    with open(os.path.join(datadir, nm["edges"]), "w") as f:
        rows = []
        for j in range(mg.Ne):
            r = "%d %d %d %d %d " % (mg.edges[j, 0], mg.edges[j, 1], mg.mark[j], mg.grad[j, 0], mg.grad[j, 1])
            if with_edge_id:
                r += "%d " % mg.edge_id[j]
            rows.append(r + "\n")
        f.write("".join(rows))
    with open(os.path.join(datadir, nm["cells"]), "w") as f:
        rows = []
        for j in range(mg.Nc):
            nf = int(mg.nfaces[j])
            r = ("%d " % nf) if with_nfaces else ""
            r += "%e %e " % (mg.xv[j], mg.yv[j])
            r += "".join("%d " % c for c in mg.cells[j, :nf])
            r += "".join("%d " % c for c in mg.neigh[j, :nf])
            rows.append(r + "\n")
        f.write("".join(rows))


# ----------------------------------------------------------------------------
# field output and restart
# ----------------------------------------------------------------------------
def write_2d(fobj, x: np.ndarray) -> None:
    """Write2DData without merging (main/physio.c:29-57): Nc doubles."""
    np.ascontiguousarray(x, dtype=F64).tofile(fobj)


def plane_layout(x: np.ndarray, Nk: np.ndarray, Nkmax: int, extra: int = 0) -> np.ndarray:
    """[Nkmax, Nc] planes of a ragged per-cell field whose rows hold Nk + extra
    values, EMPTY below each column's Nk (Write3DData, main/physio.c:66-105)."""
    Nk = np.asarray(Nk, dtype=np.int64)
    Nc = Nk.size
    off = _jagged(Nk + extra)
    out = np.full((Nkmax, Nc), EMPTY, dtype=F64)
    cell = np.repeat(np.arange(Nc), Nk)
    k = np.arange(int(Nk.sum())) - np.repeat(_jagged(Nk)[:-1], Nk)
    out[k, cell] = np.asarray(x, dtype=F64)[off[cell] + k]
    return out


def write_3d(fobj, x: np.ndarray, Nk: np.ndarray, Nkmax: int, extra: int = 0) -> None:
    """Write3DData without merging: Nkmax planes of Nc doubles, EMPTY below Nk.
    ``extra`` = 1 for fields stored with Nk+1 levels (w); the bottom face is
    not written, as in the reference."""
    plane_layout(x, Nk, Nkmax, extra).tofile(fobj)


def read_3d(fobj, Nk: np.ndarray, Nkmax: int) -> np.ndarray:
    """Read one Write3DData record back into ragged (Nk per cell) storage."""
    Nk = np.asarray(Nk, dtype=np.int64)
    Nc = Nk.size
    planes = np.fromfile(fobj, dtype=F64, count=Nkmax * Nc)
    if planes.size != Nkmax * Nc:
        raise ValueError("3-D record is short")
    planes = planes.reshape(Nkmax, Nc)
    cell = np.repeat(np.arange(Nc), Nk)
    k = np.arange(int(Nk.sum())) - np.repeat(_jagged(Nk)[:-1], Nk)
    return planes[k, cell].copy()


# The restart record (main/physio.c:343-393 / 407-483), in file order.  Each
# entry: name, rows ("cell" Nk, "edge" Nke, "cellw" Nk+1, "h" one per cell),
# and whether it is written only when turbmodel >= 1.
STORE_LAYOUT = (
    ("h", "h", False),
    ("Cn_U", "edge", False), ("Cn_U2", "edge", False),
    ("Cn_W", "cell", False), ("Cn_W2", "cell", False),
    ("Cn_R", "cell", False), ("Cn_T", "cell", False),
    ("Cn_q", "cell", True), ("Cn_l", "cell", True), ("qT", "cell", True), ("lT", "cell", True),
    ("nu_tv", "cell", False), ("kappa_tv", "cell", False),
    ("u", "edge", False), ("w", "cellw", False), ("q", "cell", False), ("qc", "cell", False),
    ("s", "cell", False), ("T", "cell", False), ("s0", "cell", False),
)


def _store_sizes(Nk: np.ndarray, Nke: np.ndarray, turbmodel: int):
    n3, ne3, Nc = int(np.sum(Nk)), int(np.sum(Nke)), int(np.size(Nk))
    size = {"h": Nc, "edge": ne3, "cell": n3, "cellw": n3 + Nc}
    return [(name, size[rows]) for name, rows, turb in STORE_LAYOUT if turbmodel >= 1 or not turb]


def store_nbytes(Nk: np.ndarray, Nke: np.ndarray, turbmodel: int = 0) -> int:
    return 4 + 8 * sum(n for _, n in _store_sizes(Nk, Nke, turbmodel))


def write_store(path: str, n: int, fields: Dict[str, np.ndarray], Nk: np.ndarray, Nke: np.ndarray,
                turbmodel: int = 0) -> None:
    """Write a restart file: the step number (int32) then the fields of
    STORE_LAYOUT in order, each as its reference rows laid end to end (which
    is the flat ragged storage used throughout this package).  A missing
    field is written as zeros."""
    with open(path, "wb") as f:
        np.array([n], dtype=I32).tofile(f)
        for name, size in _store_sizes(Nk, Nke, turbmodel):
            x = fields.get(name)
            x = np.zeros(size, dtype=F64) if x is None else np.ascontiguousarray(x, dtype=F64)
            if x.size != size:
                raise ValueError(f"store field {name}: {x.size} values, expected {size}")
            x.tofile(f)


def read_store(path: str, Nk: np.ndarray, Nke: np.ndarray, turbmodel: int = 0):
    """Read a restart file written by the reference (or `write_store`): returns
    (nstart, {name: flat ragged array})."""
    with open(path, "rb") as f:
        hdr = np.fromfile(f, dtype=I32, count=1)
        if hdr.size != 1:
            raise ValueError(f"{path}: empty restart file")
        out = {}
        for name, size in _store_sizes(Nk, Nke, turbmodel):
            x = np.fromfile(f, dtype=F64, count=size)
            if x.size != size:
                raise ValueError(f"{path}: restart file ends in field {name}")
            out[name] = x
        if f.read(1):
            raise ValueError(f"{path}: restart file is longer than the grid's record "
                             f"(turbmodel {turbmodel})")
    return int(hdr[0]), out
