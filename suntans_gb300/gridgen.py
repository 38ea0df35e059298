"""Seeded synthetic SUNTANS grids and right-hand sides.

No dataset is involved anywhere: every grid here is built from a seed, with
the shapes, sizes and value distributions of the workloads the elliptic solves
are measured on.

* `quad_channel`      structured quadrilateral channel (maxfaces 4), flat bottom.
* `delaunay_seamount` Delaunay triangulation of uniform random points in a
                      rectangle, depth ``H0 - A*exp(-r^2/(2 sigma^2))`` with
                      partial-cell z-levels stretched downward.
* `make_q_problem`    pressure right-hand side = the discrete divergence of a
                      seeded face-normal velocity, as ComputeQSource forms it
                      (main/phys.c:2364-2394; w = 0), with ``D = df/dg``.
* `make_h_problem`    free-surface right-hand side ``Ac * eta`` from a seeded
                      perturbation, ``D = sum_k dzf`` (UPredictor with E = 1,
                      main/phys.c:2935-2937).

Cells are ordered along a Morton (Z-order) curve of their centres so that
neighbouring columns sit close together in memory.  Voronoi points are cell
centroids (the reference's CorrectVoronoi with VoronoiRatio = 1,
main/grid.c:3735-3821, applied to every edge), which keeps ``dg`` away from zero
on random triangulations.
"""
from __future__ import annotations

import os

import numpy as np

from .grid import SunGrid, QProblem, HProblem, F64, I32


# ----------------------------------------------------------------------------
# vertical grid
# ----------------------------------------------------------------------------
def layer_thicknesses(maxdepth: float, Nkmax: int, rstretch: float) -> np.ndarray:
    """z-level thicknesses growing downward by ``rstretch`` and summing to ``maxdepth``."""
    if rstretch == 1.0:
        return np.full(Nkmax, maxdepth / Nkmax, dtype=F64)
    r = float(rstretch)
    dz0 = maxdepth * (r - 1.0) / (r ** Nkmax - 1.0)
    return dz0 * r ** np.arange(Nkmax, dtype=F64)


def vertical_columns(depth: np.ndarray, dz: np.ndarray, stairstep: bool, dzsmall: float = 0.1):
    """Nk per cell and the bottom-cell thickness (partial cells unless stairstep)."""
    zb = np.cumsum(dz)                     # bottom of each layer
    Nkmax = dz.size
    Nk = np.searchsorted(zb, depth * (1 - 1e-12), side="left") + 1
    Nk = np.clip(Nk, 1, Nkmax).astype(I32)
    top_of_bottom = np.where(Nk > 1, zb[np.maximum(Nk - 2, 0)], 0.0)
    if stairstep:
        dbot = dz[Nk - 1].copy()
    else:
        dbot = depth - top_of_bottom
        dbot = np.maximum(dbot, dzsmall * dz[Nk - 1])
    return Nk, dbot


def build_dzz(Nk, dz, dbot, ctop, h):
    """Ragged dzz: full layers, partial bottom, free surface in the top wet cell.

    Layers above ctop are dry (thickness 0).  The top wet cell's thickness is
    its nominal thickness plus ``h``, the free-surface height above that
    layer's top (clipped to 40% of the layer), as UpdateDZ leaves it
    (main/phys.c:816-900)."""
    Nc = Nk.size
    coff = np.zeros(Nc + 1, dtype=np.int64)
    np.cumsum(Nk, out=coff[1:])
    n3 = int(coff[-1])
    cell = np.repeat(np.arange(Nc), Nk)
    k = np.arange(n3) - coff[cell]
    dzz = dz[k].copy()
    last = coff[1:] - 1
    dzz[last] = dbot
    dzz[k < ctop[cell]] = 0.0
    top_idx = coff[:-1] + ctop
    t = dzz[top_idx]
    dzz[top_idx] = t + np.clip(h, -0.4 * t, 0.4 * t)
    return dzz


# ----------------------------------------------------------------------------
# horizontal connectivity
# ----------------------------------------------------------------------------
def _edges_from_cells(cells: np.ndarray, nfaces: np.ndarray, maxfaces: int):
    """Unique edges, grad, face/neigh/normal arrays from per-cell node lists."""
    Nc = cells.shape[0]
    fidx = np.arange(maxfaces)[None, :]
    valid = fidx < nfaces[:, None]
    a = cells
    b = np.take_along_axis(cells, (fidx + 1) % nfaces[:, None], axis=1)
    lo = np.minimum(a, b)[valid].astype(np.int64)
    hi = np.maximum(a, b)[valid].astype(np.int64)
    key = lo * (int(cells.max()) + 1) + hi
    cellof = np.repeat(np.arange(Nc), nfaces)
    slot = np.nonzero(valid.ravel())[0]
    uniq, inv = np.unique(key, return_inverse=True)
    Ne = uniq.size
    order = np.argsort(inv, kind="stable")
    inv_sorted = inv[order]
    first = np.ones(order.size, dtype=bool)
    first[1:] = inv_sorted[1:] != inv_sorted[:-1]
    grad = -np.ones((Ne, 2), dtype=I32)
    grad[inv_sorted[first], 0] = cellof[order[first]]
    second = ~first
    grad[inv_sorted[second], 1] = cellof[order[second]]
    enodes = np.zeros((Ne, 2), dtype=np.int64)
    enodes[inv, 0] = lo
    enodes[inv, 1] = hi
    face = -np.ones(Nc * maxfaces, dtype=I32)
    face[slot] = inv
    neigh = -np.ones(Nc * maxfaces, dtype=I32)
    normal = np.zeros(Nc * maxfaces, dtype=I32)
    g0 = grad[inv, 0]
    g1 = grad[inv, 1]
    other = np.where(g0 == cellof, g1, g0)
    neigh[slot] = other
    normal[slot] = np.where(g0 == cellof, 1, -1)
    return Ne, grad, enodes, face, neigh, normal


def _morton_order(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0xFFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
        return v
    xs = (x - x.min()) / max(np.ptp(x), 1e-30) * 65535
    ys = (y - y.min()) / max(np.ptp(y), 1e-30) * 65535
    code = spread(xs) | (spread(ys) << np.uint64(1))
    return np.argsort(code, kind="stable")


def _assemble(points, cells, nfaces, maxfaces, depth_fn, Nkmax, rstretch, stairstep,
              rng, name, h_sigma=0.0, ctop_frac=0.0, ctop_max=3, open_x0=False, maxdepth=None):
    Nc = cells.shape[0]
    # cell centroids (Voronoi points, VoronoiRatio = 1) and areas
    px = points[:, 0][cells]
    py = points[:, 1][cells]
    m = np.arange(maxfaces)[None, :] < nfaces[:, None]
    px = np.where(m, px, 0.0)
    py = np.where(m, py, 0.0)
    nxt = (np.arange(maxfaces)[None, :] + 1) % nfaces[:, None]
    qx = np.take_along_axis(points[:, 0][cells], nxt, 1)
    qy = np.take_along_axis(points[:, 1][cells], nxt, 1)
    cross = np.where(m, px * qy - qx * py, 0.0)
    Ac = 0.5 * cross.sum(1)
    if np.any(Ac <= 0):
        raise ValueError("cells must be counter-clockwise with positive area")
    xv = px.sum(1) / nfaces
    yv = py.sum(1) / nfaces

    # spatial ordering of cells
    perm = _morton_order(xv, yv)
    cells, nfaces, Ac, xv, yv = cells[perm], nfaces[perm], Ac[perm], xv[perm], yv[perm]

    Ne, grad, enodes, face, neigh, normal = _edges_from_cells(cells, nfaces, maxfaces)
    # order edges by the Morton rank of their first cell, for locality of dzf
    eorder = np.lexsort((grad[:, 1], grad[:, 0]))
    einv = np.empty(Ne, dtype=np.int64)
    einv[eorder] = np.arange(Ne)
    grad, enodes = grad[eorder], enodes[eorder]
    face = np.where(face >= 0, einv[np.maximum(face, 0)], -1).astype(I32)

    e0, e1 = enodes[:, 0], enodes[:, 1]
    df = np.hypot(points[e0, 0] - points[e1, 0], points[e0, 1] - points[e1, 1])
    interior = grad[:, 1] >= 0
    g0, g1 = grad[:, 0], np.maximum(grad[:, 1], 0)
    dg = np.hypot(xv[g0] - xv[g1], yv[g0] - yv[g1])
    mx = 0.5 * (points[e0, 0] + points[e1, 0])
    my = 0.5 * (points[e0, 1] + points[e1, 1])
    dgb = 2.0 * np.hypot(xv[g0] - mx, yv[g0] - my)
    dg = np.where(interior, dg, dgb)

    # vertical structure
    depth = depth_fn(xv, yv)
    md = float(depth.max()) if maxdepth is None else float(maxdepth)
    dz = layer_thicknesses(md, Nkmax, rstretch)
    Nk, dbot = vertical_columns(depth, dz, stairstep)
    ctop = np.zeros(Nc, dtype=I32)
    if ctop_frac > 0:
        sel = rng.random(Nc) < ctop_frac
        ctop[sel] = rng.integers(0, ctop_max + 1, size=int(sel.sum()))
        ctop = np.minimum(ctop, Nk - 1).astype(I32)
    h = rng.normal(0.0, h_sigma, size=Nc) if h_sigma > 0 else np.zeros(Nc)
    dzz = build_dzz(Nk, dz, dbot, ctop, h)

    Nke = np.where(interior, np.minimum(Nk[g0], Nk[g1]), Nk[g0]).astype(I32)
    coff = np.zeros(Nc + 1, dtype=np.int64)
    np.cumsum(Nk, out=coff[1:])
    eoff = np.zeros(Ne + 1, dtype=np.int64)
    np.cumsum(Nke, out=eoff[1:])
    edge = np.repeat(np.arange(Ne), Nke)
    k = np.arange(int(eoff[-1])) - eoff[edge]
    z0 = dzz[coff[g0[edge]] + k]
    z1 = np.where(interior[edge], dzz[coff[g1[edge]] + np.minimum(k, Nk[g1[edge]] - 1)], z0)
    bottom = k == Nke[edge] - 1
    # SetFluxHeight with u = 0: UpWind -> Max(dz1,dz2); bottom face -> Min (util.c:219-232)
    dzf = np.where(bottom, np.minimum(z0, z1), np.maximum(z0, z1))

    # computational cells first, then type-3 (open) boundary cells
    celltype = np.zeros(Nc, dtype=I32)
    if open_x0:
        xmin = points[:, 0].min()
        on_left = (np.abs(points[e0, 0] - xmin) < 1e-9) & (np.abs(points[e1, 0] - xmin) < 1e-9) & ~interior
        celltype[g0[on_left]] = 1
    mark = np.where(interior, 0, 1).astype(I32)
    if open_x0:
        mark[on_left] = 3
    comp = np.nonzero(celltype == 0)[0]
    bdy = np.nonzero(celltype == 1)[0]
    cellp = np.concatenate([comp, bdy]).astype(I32)
    celldist = np.array([0, comp.size, Nc], dtype=I32)

    g = SunGrid(Nc=Nc, Ne=Ne, maxfaces=maxfaces, Nkmax=Nkmax, nfaces=nfaces, neigh=neigh, face=face,
                Nk=Nk, Nke=Nke, ctop=ctop, cellp=cellp, celldist=celldist, Ac=Ac, df=df, dg=dg,
                dzz=dzz, dzf=dzf, normal=normal, grad=grad.ravel(), xv=xv, yv=yv, dz=dz, dv=depth,
                xp=np.ascontiguousarray(points[:, 0], dtype=F64), yp=np.ascontiguousarray(points[:, 1], dtype=F64),
                cnodes=np.where(np.arange(maxfaces)[None, :] < nfaces[:, None], cells, -1).astype(I32).ravel(),
                enodes=enodes.astype(I32).ravel(), mark=mark, name=name)
    return g


def from_main_grid(mg, Nkmax=10, depth_fn=None, rstretch=1.0, stairstep=False, seed=0, name="main", h_sigma=0.0,
                   ctop_frac=0.0, scale=1.0):
    """A solver grid on an input triangulation read from the model's files
    (`formats.read_main_grid`): its nodes and each cell's node list, with the
    geometry (areas, centroid Voronoi points, edge lengths and distances,
    normals) and the z-level columns built as for the synthetic grids.  Cells
    listed clockwise are reversed; the files' own edge list is not needed.
    depth_fn(x, y) defaults to a Gaussian bump over the domain (10-60 m);
    `scale` multiplies the node coordinates (cell size against depth sets how
    strongly the columns couple)."""
    points = float(scale) * np.stack([np.asarray(mg.xp, dtype=F64), np.asarray(mg.yp, dtype=F64)], axis=1)
    nfaces = np.asarray(mg.nfaces, dtype=I32)
    cells = np.array(mg.cells, dtype=np.int64, copy=True)
    mf = int(mg.maxfaces)
    fidx = np.arange(mf)[None, :]
    m = fidx < nfaces[:, None]
    c0 = np.where(m, cells, 0)
    nxt = np.take_along_axis(c0, (fidx + 1) % nfaces[:, None], axis=1)
    cross = np.where(m, points[c0, 0] * points[nxt, 1] - points[nxt, 0] * points[c0, 1], 0.0).sum(1)
    for j in np.nonzero(cross < 0)[0]:
        cells[j, :nfaces[j]] = cells[j, :nfaces[j]][::-1]
    if depth_fn is None:
        x0, x1, y0, y1 = points[:, 0].min(), points[:, 0].max(), points[:, 1].min(), points[:, 1].max()
        sig = 0.25 * max(x1 - x0, y1 - y0)
        xc, yc = 0.5 * (x0 + x1), 0.5 * (y0 + y1)
        depth_fn = lambda x, y: 60.0 - 50.0 * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / (2 * sig * sig))
    rng = np.random.default_rng(seed)
    return _assemble(points, cells, nfaces, mf, depth_fn, Nkmax, rstretch, stairstep, rng, name, h_sigma=h_sigma,
                     ctop_frac=ctop_frac)


def quad_channel(nx=64, ny=16, dx=10.0, dy=10.0, depth=20.0, Nkmax=32, rstretch=1.0, seed=0,
                 h_sigma=0.0, ctop_frac=0.0, open_x0=False, depth_fn=None, stairstep=True):
    """Structured quad channel (maxfaces 4), cells (ix, iy) counter-clockwise."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(nx + 1) * dx, np.arange(ny + 1) * dy, indexing="xy")
    points = np.stack([X.ravel(), Y.ravel()], 1)
    pid = lambda ix, iy: iy * (nx + 1) + ix
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ix, iy = ix.ravel(), iy.ravel()
    cells = np.stack([pid(ix, iy), pid(ix + 1, iy), pid(ix + 1, iy + 1), pid(ix, iy + 1)], 1)
    nfaces = np.full(cells.shape[0], 4, dtype=I32)
    dfn = depth_fn if depth_fn is not None else (lambda x, y: np.full_like(x, depth))
    return _assemble(points, cells, nfaces, 4, dfn, Nkmax, rstretch, stairstep, rng,
                     name=f"quad{nx}x{ny}x{Nkmax}", h_sigma=h_sigma, ctop_frac=ctop_frac,
                     open_x0=open_x0, maxdepth=None if depth_fn is None else None)


def hybrid_channel(nx=12, ny=6, dx=10.0, Nkmax=8, split_every=3, seed=0, h_sigma=0.0, ctop_frac=0.0,
                   depth_fn=None, open_x0=False):
    """A quad channel with every `split_every`-th quad (in a diagonal pattern)
    split into two triangles: maxfaces 4 with cells of 3 and 4 faces."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(nx + 1) * dx, np.arange(ny + 1) * dx, indexing="xy")
    pts = np.stack([X.ravel(), Y.ravel()], 1)
    cells, nf = [], []
    for iy in range(ny):
        for ix in range(nx):
            a, b = iy * (nx + 1) + ix, iy * (nx + 1) + ix + 1
            c, d = (iy + 1) * (nx + 1) + ix + 1, (iy + 1) * (nx + 1) + ix
            if (ix + iy) % split_every == 0:
                cells += [[a, b, c, a], [a, c, d, a]]
                nf += [3, 3]
            else:
                cells.append([a, b, c, d])
                nf.append(4)
    dfn = depth_fn if depth_fn is not None else (lambda x, y: 6.0 + 0.1 * x)
    return _assemble(pts, np.array(cells), np.array(nf, dtype=I32), 4, dfn, Nkmax, 1.0, False, rng,
                     name=f"hybrid{nx}x{ny}x{Nkmax}", h_sigma=h_sigma, ctop_frac=ctop_frac, open_x0=open_x0)


def seamount_depth(Lx, Ly, H0=50.0, amp=30.0, sigma=2000.0):
    def f(x, y):
        r2 = (x - 0.5 * Lx) ** 2 + (y - 0.5 * Ly) ** 2
        return H0 - amp * np.exp(-r2 / (2.0 * sigma ** 2))
    return f


def delaunay_seamount(npoints=200_000, Lx=20_000.0, Ly=10_000.0, Nkmax=50, rstretch=1.02, seed=1,
                      H0=50.0, amp=30.0, sigma=2000.0, h_sigma=0.0, ctop_frac=0.0,
                      open_x0=False, stairstep=False, corners=True):
    """Delaunay triangulation of seeded uniform random points with a Gaussian seamount."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    pts = rng.random((npoints, 2)) * np.array([Lx, Ly])
    if corners:
        pts = np.concatenate([pts, np.array([[0, 0], [Lx, 0], [Lx, Ly], [0, Ly]], dtype=F64)])
    tri = Delaunay(pts)
    cells = tri.simplices.astype(np.int64)
    # counter-clockwise orientation
    p = pts[cells]
    cr = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    flip = cr < 0
    cells[flip] = cells[flip][:, [0, 2, 1]]
    # drop degenerate slivers (zero area) that qhull can emit on hull corners
    p = pts[cells]
    cr = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    cells = cells[cr > 1e-9 * Lx * Ly / max(npoints, 1)]
    nfaces = np.full(cells.shape[0], 3, dtype=I32)
    return _assemble(pts, cells, nfaces, 3, seamount_depth(Lx, Ly, H0, amp, sigma), Nkmax, rstretch,
                     stairstep, rng, name=f"delaunay{npoints}x{Nkmax}", h_sigma=h_sigma,
                     ctop_frac=ctop_frac, open_x0=open_x0, maxdepth=H0)


# ----------------------------------------------------------------------------
# right-hand sides
# ----------------------------------------------------------------------------
def make_q_problem(g: SunGrid, seed=0, sigma_u=0.05, dt=1.0, q0_sigma=0.0) -> QProblem:
    """Divergence right-hand side (ComputeQSource, main/phys.c:2364-2394, w = 0)."""
    rng = np.random.default_rng(seed)
    eoff = g.eoff
    coff = g.coff
    interior = g.grad.reshape(-1, 2)[:, 1] >= 0
    u = rng.normal(0.0, sigma_u, size=int(eoff[-1]))
    u[np.repeat(~interior, g.Nke)] = 0.0            # closed walls carry no flux
    src = np.zeros(g.n3, dtype=F64)
    mf = g.maxfaces
    for nf in range(mf):
        cells = np.nonzero(g.nfaces > nf)[0]
        ne = g.face[cells * mf + nf]
        nrm = g.normal[cells * mf + nf].astype(F64)
        for_cells_k0 = g.ctop[cells]
        nk = g.Nke[ne] - for_cells_k0
        ok = nk > 0
        cells, ne, nrm, for_cells_k0, nk = cells[ok], ne[ok], nrm[ok], for_cells_k0[ok], nk[ok]
        rep = np.repeat(np.arange(cells.size), nk)
        kk = np.arange(int(nk.sum())) - np.repeat(np.cumsum(nk) - nk, nk) + for_cells_k0[rep]
        eidx = eoff[ne[rep]] + kk
        contrib = u[eidx] * g.dzf[eidx] * nrm[rep] * g.df[ne[rep]]
        np.add.at(src, coff[cells[rep]] + kk, contrib)
    src /= dt
    # only computational cells carry a source (ComputeQSource zeroes all, fills computational)
    mask = g.active_mask()
    src[~mask] = 0.0
    D = g.df / g.dg
    q = np.zeros(g.n3, dtype=F64)
    if q0_sigma > 0:
        q[mask] = rng.normal(0.0, q0_sigma, size=int(mask.sum()))
    c = np.ones(g.n3, dtype=F64)
    return QProblem(grid=g, D=D, src=src, q=q, c=c)


def make_h_problem(g: SunGrid, seed=0, sigma_eta=0.01, bdy_sigma=0.01) -> HProblem:
    """Free-surface right-hand side Ac*eta with D = sum_k dzf (E = 1)."""
    rng = np.random.default_rng(seed)
    eta = rng.normal(0.0, sigma_eta, size=g.Nc)
    htmp = g.Ac * eta
    h = np.zeros(g.Nc, dtype=F64)
    bdy = g.cellp[g.celldist[1]:g.celldist[2]]
    h[bdy] = rng.normal(0.0, bdy_sigma, size=bdy.size)
    htmp[bdy] = 0.0
    D = np.add.reduceat(g.dzf, g.eoff[:-1]) if g.Ne > 0 else np.zeros(0)
    return HProblem(grid=g, D=np.ascontiguousarray(D, dtype=F64), htmp=htmp, h=h)


# ----------------------------------------------------------------------------
# families of problems for the batched and serving workloads
# ----------------------------------------------------------------------------
CELL_AREA = 500.0   # m^2 per triangle, as in the 200k-point, 20 km x 10 km seamount grid


def bump_grid(nc_target: int, Nkmax: int, seed: int, aspect: float = 2.0, H0: float = 60.0, amp: float = 50.0,
              rstretch: float = 1.02):
    """Delaunay grid of ~nc_target triangles in an aspect:1 rectangle with a
    centred Gaussian bump (depth H0 - amp at the top, H0 far away)."""
    npts = max(8, int(nc_target) // 2)
    Ly = float(np.sqrt(CELL_AREA * nc_target / aspect))
    Lx = aspect * Ly
    return delaunay_seamount(npts, Lx, Ly, Nkmax=Nkmax, rstretch=rstretch, seed=seed, H0=H0, amp=amp,
                             sigma=Lx / 6.0, h_sigma=0.01)


def _batch_instance(args):
    nc, nkmax, gseed, qseeds = args
    g = bump_grid(nc, nkmax, seed=gseed)
    return [make_q_problem(g, seed=q, sigma_u=0.05, dt=20.0) for q in qseeds]


def _build_all(params, workers):
    """Builds the problems of `params` (in order), in `workers` spawned processes
    when > 1 (None: one per core, at most 16).  The calling program must be a
    file (spawned workers re-import it)."""
    if workers is None:
        workers = min(16, os.cpu_count() or 1)
    if workers <= 1 or len(params) <= 1:
        return [_batch_instance(a) for a in params]
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(workers, len(params))) as pool:
        return pool.map(_batch_instance, params, chunksize=1)


def batch_instances(n=256, seed=4, nc_range=(2000, 50000), nkmax_choices=(10, 20, 40), workers=1):
    """Independent problems with Nc log-uniform in nc_range and Nkmax drawn from
    nkmax_choices, each with its own seeded divergence right-hand side.  The
    seeds are drawn in order from `seed`, so the set does not depend on workers."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(nc_range[0]), np.log(nc_range[1])
    params = []
    for k in range(n):
        nc = int(np.exp(rng.uniform(lo, hi)))
        nkmax = int(rng.choice(nkmax_choices))
        gseed = int(rng.integers(1 << 30))
        params.append((nc, nkmax, gseed, [int(rng.integers(1 << 30))]))
    return [r[0] for r in _build_all(params, workers)]


def serving_pool(n=24, seed=5, nc_range=(1000, 200000), nkmax_range=(10, 60), rhs_per_grid=2, workers=1):
    """A pool of seeded grids (Nc log-uniform, Nkmax uniform) with a few
    seeded right-hand sides each; requests draw (grid, rhs) pairs from it."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(nc_range[0]), np.log(nc_range[1])
    params = []
    for k in range(n):
        nc = int(np.exp(rng.uniform(lo, hi)))
        nkmax = int(rng.integers(nkmax_range[0], nkmax_range[1] + 1))
        gseed = int(rng.integers(1 << 30))
        params.append((nc, nkmax, gseed, [int(rng.integers(1 << 30)) for _ in range(rhs_per_grid)]))
    return _build_all(params, workers)


def make_step_fields(g: SunGrid, seed=0, sigma_u=0.05, sigma_w=0.002, sigma_q=0.01) -> "StepFields":
    """Seeded fields for the pressure step around CGSolveQ: u*, w* and their
    previous values, the total pressure q, a zero correction qc.  Computational
    edges are the interior edges (two cells); an edge's top wet level is the
    deeper of its cells' tops."""
    from .grid import StepFields
    rng = np.random.default_rng(seed)
    grad = g.grad.reshape(g.Ne, 2)
    interior = (grad[:, 0] >= 0) & (grad[:, 1] >= 0)
    ct = g.ctop
    etop = np.where(interior, np.maximum(ct[np.maximum(grad[:, 0], 0)], ct[np.maximum(grad[:, 1], 0)]),
                    ct[np.maximum(grad[:, 0], 0)])
    etop = np.minimum(etop, np.maximum(g.Nke - 1, 0)).astype(np.int32)
    ne3 = int(g.Nke.sum())
    eoff = g.eoff
    lev = np.arange(ne3) - np.repeat(eoff[:-1], g.Nke)
    wet_e = lev >= np.repeat(etop, g.Nke)
    u = np.where(wet_e, rng.normal(0.0, sigma_u, ne3), 0.0)
    utmp2 = np.where(wet_e, rng.normal(0.0, sigma_u, ne3), 0.0)
    nw = int((g.Nk + 1).sum())
    woff = np.zeros(g.Nc + 1, dtype=np.int64)
    np.cumsum(g.Nk + 1, out=woff[1:])
    wlev = np.arange(nw) - np.repeat(woff[:-1], g.Nk + 1)
    wet_w = wlev >= np.repeat(ct, g.Nk + 1)
    w = np.where(wet_w, rng.normal(0.0, sigma_w, nw), 0.0)
    wtmp2 = np.where(wet_w, rng.normal(0.0, sigma_w, nw), 0.0)
    clev = np.arange(g.n3) - np.repeat(g.coff[:-1], g.Nk)
    wet_c = clev >= np.repeat(ct, g.Nk)
    q = np.where(wet_c, rng.normal(0.0, sigma_q, g.n3), 0.0)
    edgep = np.nonzero(interior)[0].astype(np.int32)
    return StepFields(grid=g, u=u, utmp2=utmp2, w=w, wtmp2=wtmp2, q=q, qc=np.zeros(g.n3), c=np.ones(g.n3),
                      etop=etop, edgep=edgep, edgedist=np.array([0, edgep.size], dtype=np.int32))


def make_vgrid_fields(g: SunGrid, seed=0, sigma_h=None, smoothbot=0.0, dzsmall=0.1) -> "VGridFields":
    """Seeded inputs of UpdateDZ / SetFluxHeight: a free surface that moves
    some cells' top level (N(0, sigma_h), default half the top layer), an edge
    velocity with exact zeros on some levels (UpWind's third branch), dzbot =
    the bottom cells' thickness, Nkc = the deeper of an edge's two cells."""
    from .grid import VGridFields
    rng = np.random.default_rng(seed)
    sig = 0.5 * float(g.dz[0]) if sigma_h is None else sigma_h
    h = rng.normal(0.0, sig, g.Nc)
    ne3 = int(g.Nke.sum())
    u = rng.normal(0.0, 0.05, ne3)
    u[rng.random(ne3) < 0.05] = 0.0
    last = g.coff[1:] - 1
    dzbot = g.dzz[last].copy()
    grad = g.grad.reshape(g.Ne, 2)
    c0, c1 = grad[:, 0], grad[:, 1]
    nk0 = g.Nk[np.where(c0 >= 0, c0, c1)]
    nk1 = g.Nk[np.where(c1 >= 0, c1, c0)]
    Nkc = np.maximum(np.maximum(nk0, nk1), g.Nke).astype(np.int32)
    st = make_step_fields(g, seed=seed + 1)
    return VGridFields(grid=g, h=h, u=u, dzbot=dzbot, Nkc=Nkc, smoothbot=float(smoothbot), dzsmall=float(dzsmall),
                       ctop=g.ctop.copy(), etop=st.etop.copy(), dzz=g.dzz.copy())


def edge_normals(g: SunGrid):
    """Unit normal of each edge pointing from grad[0] towards grad[1] (outward
    on boundary edges), from the plan-view geometry (gridT.n1, n2)."""
    grad = g.grad.reshape(g.Ne, 2)
    en = g.enodes.reshape(g.Ne, 2)
    x0, y0 = g.xp[en[:, 0]], g.yp[en[:, 0]]
    tx, ty = g.xp[en[:, 1]] - x0, g.yp[en[:, 1]] - y0
    L = np.hypot(tx, ty)
    nx, ny = ty / L, -tx / L
    c0 = grad[:, 0]
    flip = (g.xv[c0] - x0) * nx + (g.yv[c0] - y0) * ny > 0
    return np.where(flip, -nx, nx), np.where(flip, -ny, ny)


def edges_by_mark(mark: np.ndarray):
    """edgep / edgedist[6]: edges of mark 0 or 5 first, then marks 1..4
    (main/grid.c:1666-1679)."""
    comp = np.nonzero((mark == 0) | (mark == 5))[0]
    parts = [comp] + [np.nonzero(mark == m)[0] for m in range(1, 5)]
    edgep = np.concatenate(parts).astype(np.int32)
    edgedist = np.zeros(6, dtype=np.int32)
    edgedist[1:] = np.cumsum([p.size for p in parts])
    return edgep, edgedist


def make_upred_fields(g: SunGrid, seed=0, sigma_u=0.05, noslip_frac=0.2, nonlinear=1, thetaM=0.5,
                      laxWendroff_Vertical=1.0, nu=1e-6) -> "UPredFields":
    """Seeded inputs of UPredictor: u, w at step n (as the pressure step's),
    a free surface N(0, 0.3 dz[0]), an explicit horizontal source, surface
    stress, drag coefficients with a fraction of no-slip (-1) tops and bottoms
    on edges of two or more wet levels, and vertical viscosities."""
    from .grid import UPredFields
    rng = np.random.default_rng(seed)
    st = make_step_fields(g, seed=seed + 7, sigma_u=sigma_u)
    ne3 = int(g.Nke.sum())
    lev = np.arange(ne3) - np.repeat(g.eoff[:-1], g.Nke)
    wet = lev >= np.repeat(st.etop, g.Nke)
    utmp = np.where(wet, st.u + rng.normal(0.0, 0.1 * sigma_u, ne3), 0.0)
    h = rng.normal(0.0, 0.3 * float(g.dz[0]), g.Nc)
    tau_T = rng.normal(0.0, 1e-4, g.Ne)
    CdB = rng.uniform(1e-3, 5e-3, g.Ne)
    CdT = rng.uniform(0.0, 2e-3, g.Ne)
    multi = (g.Nke - st.etop) > 1
    CdB[multi & (rng.random(g.Ne) < noslip_frac)] = -1.0
    CdT[multi & (rng.random(g.Ne) < noslip_frac)] = -1.0
    nu_tv = rng.uniform(0.0, 1e-3, g.n3)
    nu_lax = rng.uniform(0.0, 1e-4, g.n3)
    mark = g.mark if g.mark is not None else np.where(g.grad.reshape(-1, 2)[:, 1] >= 0, 0, 1).astype(I32)
    bedgep, bedgedist = edges_by_mark(mark)
    n1, n2 = edge_normals(g)
    return UPredFields(grid=g, u=st.u, w=st.w, h=h, utmp=utmp, tau_T=tau_T, CdT=CdT, CdB=CdB, nu_tv=nu_tv,
                       nu_lax=nu_lax, nu=float(nu), laxWendroff_Vertical=float(laxWendroff_Vertical),
                       thetaM=float(thetaM), nonlinear=int(nonlinear), etop=st.etop, edgep=st.edgep,
                       edgedist=st.edgedist, bedgep=bedgep, bedgedist=bedgedist, mark=mark.astype(I32),
                       n1=n1, n2=n2)


def make_wpred_fields(g: SunGrid, seed=0, nonlinear=1, conserveMomentum=0, n=5, AB=3, nu=1e-6, nu_H=0.1,
                      CdW=0.002, laxWendroff_Vertical=1.0) -> "WPredFields":
    """Seeded inputs of WPredictor: w and u as the pressure step's, Adams-Bashforth
    histories, a pressure field, vertical viscosities."""
    from .grid import WPredFields
    rng = np.random.default_rng(seed)
    st = make_step_fields(g, seed=seed + 3)
    Cn_W = rng.normal(0.0, 1e-4, g.n3)
    Cn_W2 = rng.normal(0.0, 1e-4, g.n3)
    return WPredFields(grid=g, w=st.w, Cn_W=Cn_W, Cn_W2=Cn_W2, q=st.q, nu_tv=rng.uniform(0.0, 1e-3, g.n3),
                       nu_lax=rng.uniform(0.0, 1e-4, g.n3), utmp2=st.u, nu=float(nu), nu_H=float(nu_H),
                       CdW=float(CdW), laxWendroff_Vertical=float(laxWendroff_Vertical), nonlinear=int(nonlinear),
                       conserveMomentum=int(conserveMomentum), n=int(n), AB=int(AB), etop=st.etop, edgep=st.edgep,
                       edgedist=st.edgedist)
