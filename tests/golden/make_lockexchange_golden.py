"""Writes tests/golden/runs/lockexchange_cfg1.npz: the inputs and outputs of the
reference's own CGSolveQ and CGSolve over a 10-step run of the reference model
on the 64 x 16 quad lock-exchange channel (dx = dy = 10 m, flat 20 m,
Nkmax 32 uniform levels; rho' = -0.5e-3 for x < 320 m, +0.5e-3 beyond;
u = N(0, 0.01 m/s) face-velocity noise; nonhydrostatic, dt 1 s; CGSolve to
epsilon 1e-10 with hprecond 1, CGSolveQ to qepsilon 1e-10 with qprecond 1 and
resnorm 1, maxiters and qmaxiters 1000).

The reference model is built by `make -C oracle lockx` with the case
functions of oracle/lockx_case.c and its two solver call sites redirected to
oracle/lockx_dump.c, which records every solve.  This script writes the
channel's input triangulation in the reference's file formats, a suntans.dat
made from the reference's examples/lockexchange/rundata/suntans.dat with the
keys above changed, runs the reference's grid step (sun -g) and its 10 time
steps (sun -s), and stores the grid, every CGSolve and the CGSolveQ calls of
steps 1, 5 and 10 (their right-hand sides are random-looking, so storing all
ten would make the fixture large).

Needs the reference sources (SUNTANS_REFDIR or the oracle build's default).
"""
from __future__ import annotations

import os
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as om  # noqa: E402
from suntans_gb300 import formats as fm  # noqa: E402

NX, NY, DX = 64, 16, 10.0
Q_STEPS = (1, 5, 10)
OVERRIDES = {
    "Nkmax": "32", "stairstep": "1", "rstretch": "1", "CorrectVoronoi": "0", "VoronoiRatio": "0",
    "beta": "1", "theta": "0.55", "dt": "1", "nsteps": "10", "ntout": "10", "ntprog": "100", "ntconserve": "10",
    "nonhydrostatic": "1", "cgsolver": "1", "maxiters": "1000", "qmaxiters": "1000", "qprecond": "1",
    "hprecond": "1", "epsilon": "1e-10", "qepsilon": "1e-10", "resnorm": "1", "maxFaces": "4",
}


def quad_channel_main_grid():
    """The 64 x 16 channel's input triangulation: nodes (i, j) at (i dx, j dx),
    cells listed counter-clockwise from their lower-left node, faces in node
    order (bottom, right, top, left), walls on every boundary edge (mark 1)."""
    nid = lambda i, j: i * (NY + 1) + j  # noqa: E731
    cid = lambda i, j: i * NY + j if 0 <= i < NX and 0 <= j < NY else -1  # noqa: E731
    xp = np.array([i * DX for i in range(NX + 1) for j in range(NY + 1)])
    yp = np.array([j * DX for i in range(NX + 1) for j in range(NY + 1)])
    cells, neigh, xv, yv = [], [], [], []
    for i in range(NX):
        for j in range(NY):
            cells.append([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)])
            neigh.append([cid(i, j - 1), cid(i + 1, j), cid(i, j + 1), cid(i - 1, j)])
            xv.append((i + 0.5) * DX)
            yv.append((j + 0.5) * DX)
    edges, grad, mark, seen = [], [], [], {}
    for c, (nodes, nb) in enumerate(zip(cells, neigh)):
        for f in range(4):
            a, b = nodes[f], nodes[(f + 1) % 4]
            key = (min(a, b), max(a, b))
            if key in seen:
                continue
            seen[key] = len(edges)
            edges.append([a, b])
            grad.append([c, nb[f]])
            mark.append(0 if nb[f] >= 0 else 1)
    Ne = len(edges)
    return fm.MainGrid(maxfaces=4, xp=xp, yp=yp, edges=np.array(edges), mark=np.array(mark),
                       grad=np.array(grad), edge_id=np.zeros(Ne, dtype=int), nfaces=np.full(NX * NY, 4),
                       xv=np.array(xv), yv=np.array(yv), cells=np.array(cells), neigh=np.array(neigh))


def write_suntans_dat(template: str, path: str):
    """The template's lines with OVERRIDES' values (comments kept: the
    reference's GetValue ignores a one-character value that ends its line)."""
    out, done = [], set()
    for line in open(template):
        parts = line.split(None, 1)
        if parts and parts[0] in OVERRIDES:
            rest = parts[1].split(None, 1) if len(parts) > 1 else []
            comment = rest[1] if len(rest) > 1 else "# set\n"
            out.append(f"{parts[0]}\t{OVERRIDES[parts[0]]}\t{comment if comment.endswith(chr(10)) else comment + chr(10)}")
            done.add(parts[0])
        else:
            out.append(line)
    for k, v in OVERRIDES.items():
        if k not in done:
            out.append(f"{k}\t{v}\t# set\n")
    open(path, "w").write("".join(out))


def read_records(path: str):
    """The dump's arrays, in order."""
    data = open(path, "rb").read()
    off, arrays = 0, []
    while off < len(data):
        t = data[off:off + 1].decode()
        (n,) = struct.unpack_from("<i", data, off + 1)
        off += 5
        dt = np.int32 if t == "i" else np.float64
        arrays.append(np.frombuffer(data, dtype=dt, count=n, offset=off).copy())
        off += n * dt().itemsize
    return arrays


def main():
    if om.build_ref() is None:
        raise SystemExit("reference sources not found; cannot generate the lock-exchange fixture")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "lockx"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "lockx", "sun_lockx")
    template = os.path.join(om.ref_examples_dir(), "lockexchange", "rundata", "suntans.dat")
    work = tempfile.mkdtemp(prefix="lockx_")
    try:
        fm.write_main_grid(quad_channel_main_grid(), work, with_edge_id=False)
        write_suntans_dat(template, os.path.join(work, "suntans.dat"))
        for flag in ("-g", "-s"):
            r = subprocess.run([exe, flag, f"--datadir={work}"], cwd=work, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit(f"sun {flag} failed:\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        arrs = read_records(os.path.join(work, "solver_dump.bin"))
    finally:
        shutil.rmtree(work, ignore_errors=True)
    out = {}
    it = iter(arrs)
    q_seen, h_steps = 0, []
    for tag in it:
        kind, step = int(tag[0]), int(tag[1])
        if kind == 0:
            sizes, props = next(it), next(it)
            for k in ("nfaces", "neigh", "face", "Nk", "Nke", "cellp", "celldist", "Ac", "df", "dg", "xv", "yv"):
                out[k] = next(it)
            out["sizes"], out["props"] = sizes, props
        elif kind == 1:
            rec = {k: next(it) for k in ("ctop", "dzz", "dzf", "D", "q_in", "src", "q_out", "niters")}
            q_seen += 1
            if step in Q_STEPS:
                for k, v in rec.items():
                    out[f"q{step}_{k}"] = v
        else:
            rec = {k: next(it) for k in ("D", "h_in", "htmp", "h_out", "niters")}
            h_steps.append(step)
            for k, v in rec.items():
                out[f"h{step}_{k}"] = v
    if q_seen != 10 or len(h_steps) != 10:
        raise SystemExit(f"expected 10 solves of each kind, got CGSolveQ {q_seen}, CGSolve {len(h_steps)}")
    out["q_steps"] = np.array(Q_STEPS, dtype=np.int32)
    out["h_steps"] = np.array(h_steps, dtype=np.int32)
    os.makedirs(os.path.join(HERE, "runs"), exist_ok=True)
    path = os.path.join(HERE, "runs", "lockexchange_cfg1.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes; CGSolveQ iterations",
          [int(out[f"q{s}_niters"][0]) for s in Q_STEPS], "CGSolve", [int(out[f"h{s}_niters"][0]) for s in h_steps])


if __name__ == "__main__":
    main()
