"""Grid and field files in the reference's formats (suntans_gb300/formats.py).

The reference's own reader (ReadGrid, main/gridio.c:54-187) and writers
(Write2DData / Write3DData, main/physio.c:29-105), compiled from its sources
into the reference library, are the checker where that library exists: the
reference reads the files written here into the same arrays as `read_grid`,
including files with the irregular spacing and skipped fields its tokenizer
accepts, and the field writers produce the same bytes."""
import os

import numpy as np
import pytest

from oracle import oracle as om
from suntans_gb300 import formats as fm
from suntans_gb300 import gridgen as gg

# Each value is followed by a comment, as in the reference's examples: its
# GetValue (main/fileio.c:237-265) takes a value that ends its line after a
# single character for a missing one.
SUNTANS_DAT = """maxFaces {mf}	# faces per cell
Nkmax {nk}	# layers
points points.dat	# input
edges edges.dat	# input
cells cells.dat	# input
depth depth.dat	# input
nodes nodes.dat	# output
celldata celldata.dat	# output
edgedata edgedata.dat	# output
vertspace vertspace.dat	# output
topology topology.dat	# output
"""


def _grids():
    return {
        "quad": gg.quad_channel(nx=12, ny=5, Nkmax=6, open_x0=True, depth_fn=lambda x, y: 8.0 + 0.05 * x,
                                stairstep=False),
        "tri": gg.delaunay_seamount(npoints=300, Lx=2000.0, Ly=1000.0, Nkmax=9, sigma=300.0, seed=3),
    }


GRIDS = _grids()


def _round(x):
    return np.array([float("%e" % v) for v in np.ravel(x)])


def _write(tmp_path, g, tag="g"):
    d = tmp_path / tag
    gf = fm.GridFiles.from_sungrid(g)
    fm.write_grid(gf, str(d))
    (d / "suntans.dat").write_text(SUNTANS_DAT.format(mf=g.maxfaces, nk=g.Nkmax))
    return gf, str(d)


def _ref():
    if not om.available("ref"):
        pytest.skip("reference library not built here")
    return om.Oracle("ref")


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_grid_files_round_trip(tmp_path, name):
    g = GRIDS[name]
    gf, d = _write(tmp_path, g)
    rd = fm.read_grid(d, maxfaces=g.maxfaces)
    assert (rd.Nc, rd.Ne, rd.Np, rd.Nkmax) == (g.Nc, g.Ne, gf.Np, g.Nkmax)
    for f in ("nfaces", "Nk", "face", "neigh", "normal", "cells", "mnptr", "Nke", "Nkc", "grad", "gradf",
              "mark", "edges", "edge_id", "eptr", "celldist", "edgedist", "cellp", "edgep", "ppneighs",
              "peneighs", "pcneighs", "ppoff", "peoff", "pcoff", "Nkp"):
        assert np.array_equal(getattr(rd, f), getattr(gf, f)), f
    for f in ("xv", "yv", "Ac", "dv", "def_", "df", "dg", "n1", "n2", "xe", "ye", "xp", "yp", "dz"):
        assert np.array_equal(getattr(rd, f), _round(getattr(gf, f))), f
    sg = rd.to_sungrid()
    sg.validate()
    assert np.array_equal(sg.face, g.face) and np.array_equal(sg.neigh, g.neigh)
    assert sg.ncomp == g.ncomp and sg.n3 == g.n3 and np.all(sg.ctop == 0)
    assert np.array_equal(rd.computational_edges(), np.nonzero(g.mark == 0)[0])


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_reference_reads_the_files_as_read_grid_does(tmp_path, name):
    ref = _ref()
    g = GRIDS[name]
    gf, d = _write(tmp_path, g)
    ours = fm.read_grid(d, maxfaces=g.maxfaces)
    r = ref.read_grid(d)
    assert (r["Nc"], r["Ne"], r["Np"], r["maxfaces"], r["Nkmax"], r["Nneighs"]) == \
        (ours.Nc, ours.Ne, ours.Np, g.maxfaces, ours.Nkmax, 0)
    _compare_ref(r, ours)


def _compare_ref(r, ours):
    mf = ours.maxfaces
    slot = (np.arange(mf)[None, :] < ours.nfaces[:, None]).ravel()
    for f in ("face", "neigh", "normal", "cells"):
        assert np.array_equal(r[f][slot], getattr(ours, f)[slot]), f
    assert np.array_equal(r["def"][slot], ours.def_[slot])
    for f in ("nfaces", "Nk", "mnptr", "cellp", "Nke", "Nkc", "mark", "edge_id", "eptr", "edgep", "grad",
              "gradf", "celldist", "edgedist", "edges", "ppneighs", "peneighs", "pcneighs", "Nkp"):
        assert np.array_equal(r[f], getattr(ours, f)), f
    assert np.array_equal(r["localtoglobalpoints"], ours.node_id)
    for f, off in (("numppneighs", ours.ppoff), ("numpeneighs", ours.peoff), ("numpcneighs", ours.pcoff)):
        assert np.array_equal(r[f], np.diff(off)), f
    for f in ("xv", "yv", "Ac", "dv", "df", "dg", "n1", "n2", "xe", "ye", "xp", "yp", "dz", "Actotal"):
        assert np.array_equal(r[f], getattr(ours, f)), f


def _perturb(path, rng):
    """Rewrite a file with the irregular input the reference's tokenizer takes:
    tabs and repeated blanks, CR before LF, skipped fields (any character
    outside 0-9 . + - e), a leading '+', numbers with a dangling exponent
    ('1e+' reads as 1) and integer fields with a fraction (truncated)."""
    lines = open(path).read().split("\n")
    out = []
    for ln in lines:
        if not ln:
            out.append(ln)
            continue
        toks = ln.split()
        new = []
        for t in toks:
            r = rng.random()
            if r < 0.1 and "e" not in t and "." not in t and t.lstrip("-").isdigit():
                t = t + ".75" if not t.startswith("-") else t + ".25"
            elif r < 0.2 and t[0].isdigit():
                t = "+" + t
            elif r < 0.25 and t.isdigit():
                t = t + "e+"
            new.append(t)
            if rng.random() < 0.1:
                new.append("note:x")
        sep = "\t" if rng.random() < 0.5 else "   "
        out.append(sep.join(new) + ("\r" if rng.random() < 0.5 else ""))
    open(path, "w").write("\n".join(out))


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_irregular_files_read_like_the_reference(tmp_path, name):
    ref = _ref()
    g = GRIDS[name]
    gf, d = _write(tmp_path, g)
    rng = np.random.default_rng(11)
    for f in ("celldata.dat.0", "edgedata.dat.0", "nodes.dat.0", "topology.dat.0", "vertspace.dat"):
        _perturb(os.path.join(d, f), rng)
    ours = fm.read_grid(d, maxfaces=g.maxfaces)
    _compare_ref(ref.read_grid(d), ours)


def test_field_tokenizer_rules(tmp_path):
    p = tmp_path / "t.dat"
    p.write_bytes(b"1 -2.5\t+3e2 x 4.9e-1 1e+ . - e5 7abc 8\r\n1-2 .5")
    assert list(fm.read_fields(str(p))) == [1.0, -2.5, 300.0, 0.49, 1.0, 0.0, 0.0, 0.0, 8.0, 1.0, 0.5]
    assert fm.count_lines(str(p)) == 1


def test_short_file_raises(tmp_path):
    g = GRIDS["quad"]
    gf, d = _write(tmp_path, g)
    p = os.path.join(d, "edgedata.dat.0")
    s = open(p).read()
    open(p, "w").write(s[: len(s) // 2] + "\n" * (s.count("\n") - s[: len(s) // 2].count("\n")))
    with pytest.raises(ValueError):
        fm.read_grid(d, maxfaces=g.maxfaces)


def test_too_many_faces_raises(tmp_path):
    g = GRIDS["quad"]
    gf, d = _write(tmp_path, g)
    with pytest.raises(ValueError):
        fm.read_grid(d, maxfaces=3)


@pytest.mark.parametrize("extra", [0, 1])
def test_3d_output_matches_reference_bytes(tmp_path, extra):
    ref = _ref()
    g = GRIDS["tri"]
    rng = np.random.default_rng(5)
    x = rng.normal(size=int(np.sum(g.Nk + extra)))
    with open(tmp_path / "ours.dat", "wb") as f:
        fm.write_3d(f, x, g.Nk, g.Nkmax, extra)
    ref.write_3d(str(tmp_path / "ref.dat"), g.Nk, g.Nkmax, x, extra)
    a = (tmp_path / "ours.dat").read_bytes()
    assert a == (tmp_path / "ref.dat").read_bytes()
    assert len(a) == 8 * g.Nkmax * g.Nc
    if extra == 0:
        with open(tmp_path / "ours.dat", "rb") as f:
            assert np.array_equal(fm.read_3d(f, g.Nk, g.Nkmax), x)


def test_2d_output_matches_reference_bytes(tmp_path):
    ref = _ref()
    g = GRIDS["tri"]
    h = np.random.default_rng(6).normal(size=g.Nc)
    with open(tmp_path / "ours.dat", "wb") as f:
        fm.write_2d(f, h)
    ref.write_2d(str(tmp_path / "ref.dat"), h)
    assert (tmp_path / "ours.dat").read_bytes() == (tmp_path / "ref.dat").read_bytes()


def test_3d_planes_put_empty_below_the_bottom():
    Nk = np.array([1, 3, 2], dtype=np.int32)
    x = np.arange(6, dtype=float)
    P = fm.plane_layout(x, Nk, 4)
    assert P.shape == (4, 3)
    assert list(P[:, 0]) == [0, fm.EMPTY, fm.EMPTY, fm.EMPTY]
    assert list(P[:, 1]) == [1, 2, 3, fm.EMPTY]
    assert list(P[:, 2]) == [4, 5, fm.EMPTY, fm.EMPTY]


@pytest.mark.parametrize("turbmodel", [0, 1])
def test_store_round_trip_and_layout(tmp_path, turbmodel):
    g = GRIDS["quad"]
    rng = np.random.default_rng(7)
    n3, ne3 = g.n3, int(g.Nke.sum())
    fields = {"h": rng.normal(size=g.Nc), "u": rng.normal(size=ne3), "w": rng.normal(size=n3 + g.Nc),
              "q": rng.normal(size=n3), "qc": rng.normal(size=n3), "nu_tv": rng.normal(size=n3)}
    p = str(tmp_path / "store.dat.0")
    fm.write_store(p, 42, fields, g.Nk, g.Nke, turbmodel)
    assert os.path.getsize(p) == fm.store_nbytes(g.Nk, g.Nke, turbmodel)
    # reference layout: int n, h[Nc], 2 edge fields, 4 cell fields, [4 turbulence fields], nu_tv, kappa_tv,
    # u (edges), w (Nk+1 per cell), q, qc, s, T, s0  (main/physio.c:343-393)
    ncell = 4 + (4 if turbmodel else 0) + 2 + 5
    assert fm.store_nbytes(g.Nk, g.Nke, turbmodel) == 4 + 8 * (g.Nc + 3 * ne3 + ncell * n3 + n3 + g.Nc)
    n, got = fm.read_store(p, g.Nk, g.Nke, turbmodel)
    assert n == 42
    for k, v in fields.items():
        assert np.array_equal(got[k], v)
    raw = np.fromfile(p, dtype=np.uint8)
    off = 4 + 8 * (g.Nc + 2 * ne3 + (4 + (4 if turbmodel else 0) + 2) * n3)
    assert np.array_equal(np.frombuffer(raw[off:off + 8 * ne3].tobytes(), dtype=np.float64), fields["u"])
    with pytest.raises(ValueError):
        fm.read_store(p, g.Nk, g.Nke, 1 - turbmodel)


def _hybrid_grid():
    """A quad channel with every third quad split into two triangles (maxfaces 4, mixed nfaces)."""
    nx, ny, dx = 9, 4, 10.0
    X, Y = np.meshgrid(np.arange(nx + 1) * dx, np.arange(ny + 1) * dx, indexing="xy")
    pts = np.stack([X.ravel(), Y.ravel()], 1)
    pid = lambda ix, iy: iy * (nx + 1) + ix
    cells, nf = [], []
    for iy in range(ny):
        for ix in range(nx):
            a, b, c, d = pid(ix, iy), pid(ix + 1, iy), pid(ix + 1, iy + 1), pid(ix, iy + 1)
            if (ix + iy) % 3 == 0:
                cells += [[a, b, c, -1], [a, c, d, -1]]
                nf += [3, 3]
            else:
                cells.append([a, b, c, d])
                nf.append(4)
    cells = np.array(cells)
    cells = np.where(cells < 0, cells[:, :1], cells)  # padding slots are ignored past nfaces
    return gg._assemble(pts, cells, np.array(nf, dtype=np.int32), 4, lambda x, y: 6.0 + 0.1 * x, 5, 1.0, False,
                        np.random.default_rng(1), "hybrid")


def test_hybrid_grid_round_trip_and_reference(tmp_path):
    g = _hybrid_grid()
    g.validate()
    assert set(np.unique(g.nfaces)) == {3, 4}
    gf, d = _write(tmp_path, g)
    rd = fm.read_grid(d, maxfaces=4)
    assert np.array_equal(rd.nfaces, g.nfaces) and np.array_equal(rd.face, gf.face)
    assert np.array_equal(rd.neigh, gf.neigh) and np.array_equal(rd.cells, gf.cells)
    assert np.array_equal(rd.def_, _round(gf.def_))
    if om.available("ref"):
        _compare_ref(om.Oracle("ref").read_grid(d), rd)


# ---------------------------------------------------------------------------
# the input triangulation (points / edges / cells) of the reference's examples
# ---------------------------------------------------------------------------
REF_EXAMPLES = om.ref_examples_dir() or ""
# (folder, points, edges, cells, maxFaces): the grids the reference ships with its examples
MAIN_GRIDS = [
    ("riverplume/grids/tri", "points.dat", "edges.dat", "cells.dat", 3),
    ("riverplume/grids/quad", "points.dat", "edges.dat", "cells.dat", 4),
    ("riverplume/grids/hex", "points.dat", "edges.dat", "cells.dat", 7),
    ("riverplume/grids/hybrid", "points.dat", "edges.dat", "cells.dat", 7),
    ("riverplume/grids/gmsh", "points.dat", "edges.dat", "cells.dat", 4),
    ("boundaries/data-files", "points-quad.dat", "edges-quad.dat", "cells-quad.dat", 4),
    ("cylinder/data-files", "points-tri.dat", "edges-tri.dat", "cells-tri.dat", 3),
    ("cylinder/data-files", "points-quad.dat", "edges-quad.dat", "cells-quad.dat", 4),
    ("cavity/data-files", "pointsXZ.dat", "edgesXZ.dat", "cellsXZ.dat", 3),
    ("cavity/data-files", "pointsXZ-quad.dat", "edgesXZ-quad.dat", "cellsXZ-quad.dat", 4),
    ("EstuaryNetcdf/grid", "points.dat", "edges.dat", "cells.dat", 3),
    ("heatflux/rundata", "points.dat", "edges.dat", "cells.dat", 4),
]
MAIN_IDS = [f"{d}:{c}" for d, _, _, c, _ in MAIN_GRIDS]
MAIN_DAT = "maxFaces {mf}\t# faces per cell\npoints {p}\t# input\nedges {e}\t# input\ncells {c}\t# input\n" \
           "depth depth.dat\t# input\nnodes nodes.dat\t# output\ncelldata celldata.dat\t# output\n" \
           "edgedata edgedata.dat\t# output\nvertspace vertspace.dat\t# output\ntopology topology.dat\t# output\n"


def _main_case(tmp_path, case):
    d, p, e, c, mf = case
    src = os.path.join(REF_EXAMPLES, d)
    if not os.path.isfile(os.path.join(src, c)):
        pytest.skip("the reference's example grids are not present on this host")
    tmp_path.mkdir(parents=True, exist_ok=True)
    (tmp_path / "suntans.dat").write_text(MAIN_DAT.format(mf=mf, p=os.path.join(src, p), e=os.path.join(src, e),
                                                          c=os.path.join(src, c)))
    names = {"points": os.path.join(src, p), "edges": os.path.join(src, e), "cells": os.path.join(src, c)}
    return fm.read_main_grid(str(tmp_path), maxfaces=mf, names=names), str(tmp_path)


def _compare_main(r, mg):
    assert (r["Nc"], r["Ne"], r["Np"], r["maxfaces"]) == (mg.Nc, mg.Ne, mg.Np, mg.maxfaces)
    slot = (np.arange(mg.maxfaces)[None, :] < mg.nfaces[:, None]).ravel()
    assert np.array_equal(r["nfaces"], mg.nfaces)
    assert np.array_equal(r["cells"][slot], mg.cells.ravel()[slot])
    assert np.array_equal(r["neigh"][slot], mg.neigh.ravel()[slot])
    assert np.array_equal(r["edges"], mg.edges.ravel()) and np.array_equal(r["grad"], mg.grad.ravel())
    assert np.array_equal(r["mark"], mg.mark) and np.array_equal(r["edge_id"], mg.edge_id)
    for f in ("xv", "yv", "xp", "yp"):
        assert np.array_equal(r[f], getattr(mg, f)), f


@pytest.mark.parametrize("case", MAIN_GRIDS, ids=MAIN_IDS)
def test_example_grids_read_like_the_reference(tmp_path, case):
    """The grids shipped with the reference's examples (triangles, quads,
    hexagons, mixed cells up to 7 faces, with and without the nfaces and
    edge_id columns) read into the arrays the reference's ReadMainGrid fills."""
    ref = _ref()
    mg, d = _main_case(tmp_path, case)
    _compare_main(ref.read_main_grid(d), mg)


@pytest.mark.parametrize("case", [MAIN_GRIDS[0], MAIN_GRIDS[3], MAIN_GRIDS[11]], ids=[MAIN_IDS[0], MAIN_IDS[3],
                                                                                     MAIN_IDS[11]])
def test_main_grid_writers_round_trip(tmp_path, case):
    """write_main_grid's files (with and, for triangles, without the optional
    columns) are read back alike here and by the reference."""
    ref = _ref()
    mg, _ = _main_case(tmp_path / "src", case)
    variants = [(True, True), (True, False)]
    if np.all(mg.nfaces == 3):
        variants.append((False, True))
    for k, (wnf, wid) in enumerate(variants):
        d = tmp_path / f"w{k}"
        fm.write_main_grid(mg, str(d), with_nfaces=wnf, with_edge_id=wid)
        (d / "suntans.dat").write_text(MAIN_DAT.format(mf=mg.maxfaces, p="points.dat", e="edges.dat", c="cells.dat"))
        back = fm.read_main_grid(str(d), maxfaces=mg.maxfaces)
        assert np.array_equal(back.nfaces, mg.nfaces) and np.array_equal(back.cells, mg.cells)
        assert np.array_equal(back.neigh, mg.neigh) and np.array_equal(back.grad, mg.grad)
        assert np.array_equal(back.edge_id, mg.edge_id if wid else np.zeros_like(mg.edge_id))
        assert np.array_equal(back.xv, _round(mg.xv)) and np.array_equal(back.xp, _round(mg.xp))
        _compare_main(ref.read_main_grid(str(d)), back)


def test_column_count_rules(tmp_path):
    """get_num_columns counts as the reference's getNumColumns: leading blanks,
    runs of blanks, a trailing blank (taken back) and a trailing tab (not)."""
    ref = _ref()
    cases = [b"  1 2 3\n", b"1 2 3 \n", b"1\t2\t\n", b"1  2   3    4\n5 6\n", b"1 2 3 \r\n", b"7", b"\n1 2\n",
             b"\t\t1 \t2\n"]
    ref.lib.getNumColumns.restype = __import__("ctypes").c_int
    for k, data in enumerate(cases):
        f = tmp_path / f"c{k}.dat"
        f.write_bytes(data)
        assert fm.get_num_columns(str(f)) == ref.lib.getNumColumns(str(f).encode()), data


def test_main_grid_too_many_faces_raises(tmp_path):
    mg = fm.MainGrid(maxfaces=4, xp=np.zeros(4), yp=np.zeros(4), edges=np.zeros((0, 2), dtype=np.int32),
                     mark=np.zeros(0, dtype=np.int32), grad=np.zeros((0, 2), dtype=np.int32),
                     edge_id=np.zeros(0, dtype=np.int32), nfaces=np.array([4], dtype=np.int32), xv=np.zeros(1),
                     yv=np.zeros(1), cells=np.array([[0, 1, 2, 3]], dtype=np.int32),
                     neigh=-np.ones((1, 4), dtype=np.int32))
    fm.write_main_grid(mg, str(tmp_path))
    with pytest.raises(ValueError):
        fm.read_main_grid(str(tmp_path), maxfaces=3)
