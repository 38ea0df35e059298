"""Generates tests/golden/examples/*.npz: solver parity cases on grids the
reference ships with its examples, with outputs from the REFERENCE itself.

Run where the SUNTANS sources are present (the reference library is built by
`make -C oracle ref` from them; the example grids are read from the source
tree's examples/ folder):

    python tests/golden/make_example_golden.py

Each fixture holds a solver grid built from one example's input triangulation
(`formats.read_main_grid` + `gridgen.from_main_grid`: hexagons and mixed cells
of up to 7 faces, coordinates scaled by 0.02 so that cells of ~20 m couple
with columns 10-60 m deep), seeded CGSolveQ / CGSolve problems on it, and the
reference's solutions and iteration counts for qprecond 0, 1, 2 and
hprecond 0, 1.  The inputs are stored, so the check needs neither the
reference nor its example files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as om  # noqa: E402
from suntans_gb300 import formats as fm  # noqa: E402
from suntans_gb300 import gridgen as gg  # noqa: E402
from suntans_gb300.grid import SolverProps  # noqa: E402

GRID_FIELDS = ("nfaces", "neigh", "face", "Nk", "Nke", "ctop", "cellp", "celldist", "Ac", "df", "dg", "dzz", "dzf")
om.build_ref()
EXAMPLES = om.ref_examples_dir() or ""
# fixture name: (example folder, maxFaces of its suntans.dat)
CASES = {"riverplume_hex": ("riverplume/grids/hex", 7), "riverplume_hybrid": ("riverplume/grids/hybrid", 7)}


def main():
    if om.build_ref() is None:
        raise SystemExit("reference sources not found; cannot generate golden vectors")
    ref = om.Oracle("ref")
    os.makedirs(os.path.join(HERE, "examples"), exist_ok=True)
    for name, (folder, mf) in CASES.items():
        mg = fm.read_main_grid(os.path.join(EXAMPLES, folder), maxfaces=mf)
        g = gg.from_main_grid(mg, Nkmax=6, ctop_frac=0.2, h_sigma=0.1, seed=41, name=name, scale=0.02)
        g.validate()
        out = {f: getattr(g, f) for f in GRID_FIELDS}
        out["sizes"] = np.array([g.Nc, g.Ne, g.maxfaces, g.Nkmax], dtype=np.int32)
        qp = gg.make_q_problem(g, seed=42, q0_sigma=0.01)
        hp = gg.make_h_problem(g, seed=43)
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
        path = os.path.join(HERE, "examples", f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: Nc={g.Nc} faces {sorted(set(g.nfaces.tolist()))} n3={g.n3} "
              f"iters q={[int(out[f'n_qp{k}']) for k in range(3)]} h={[int(out[f'n_hp{k}']) for k in range(2)]} "
              f"{os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
