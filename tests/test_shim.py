"""The SUNTANS-side adapter: patch_phys.sh redirects exactly the two solver
call sites of a copy of main/phys.c, and the patched file plus
sgpu_suntans.c compile against the model's own headers.  Needs the SUNTANS
sources (skipped where they are absent); runs on CPU only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle import oracle as om  # noqa: E402

om.build_ref()  # records where the reference sources lie, where they are present
REF = om.ref_dir() or ""
SHIM = os.path.join(ROOT, "suntans_gb300", "shim")

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "phys.c")),
                                reason="SUNTANS sources not present on this host")


def test_patch_and_compile(tmp_path):
    phys = tmp_path / "phys.c"
    shutil.copy(os.path.join(REF, "phys.c"), phys)
    r = subprocess.run(["sh", os.path.join(SHIM, "patch_phys.sh"), str(phys)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    new = phys.read_text()
    old = open(os.path.join(REF, "phys.c")).read()
    assert new.count("sgpu_CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);") == 1
    assert new.count("sgpu_CGSolve(grid,phys,prop,myproc,numprocs,comm);") == 1
    # nothing else changed: same lines apart from the 2 declarations and the 2 calls
    diff = [a for a in new.splitlines() if "sgpu_" not in a]
    assert diff == [a for a in old.splitlines() if not a.strip().startswith(("CGSolveQ(phys->qc", "CGSolve(grid"))]
    cc = ["gcc", "-fcommon", "-DNOMPI", "-DNONETCDF", "-w", f"-I{REF}", f"-I{ROOT}/include", "-c"]
    r = subprocess.run(cc + [str(phys), "-o", str(tmp_path / "phys.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(cc + [os.path.join(SHIM, "sgpu_suntans.c"), "-o", str(tmp_path / "shim.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", str(tmp_path / "shim.o")], capture_output=True, text=True).stdout
    for s in ("sgpu_CGSolveQ", "sgpu_CGSolve", "sgpu_cgsolveq", "sgpu_cgsolve", "sgpu_create"):
        assert s in syms


def test_patch_step_mode_and_compile(tmp_path):
    """With "step", ComputeQSource and Corrector in Solve move to the adapter too."""
    phys = tmp_path / "phys.c"
    shutil.copy(os.path.join(REF, "phys.c"), phys)
    r = subprocess.run(["sh", os.path.join(SHIM, "patch_phys.sh"), str(phys), "step"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    new = phys.read_text()
    assert new.count("sgpu_ComputeQSource(phys->stmp,grid,phys,prop,myproc,numprocs);") == 1
    assert new.count("sgpu_Corrector(phys->qc,grid,phys,prop,myproc,numprocs,comm);") == 1
    assert new.count("sgpu_WPredictor(grid,phys,prop,myproc,numprocs,comm);") == 1
    old = open(os.path.join(REF, "phys.c")).read()
    diff = [a for a in new.splitlines() if "sgpu_" not in a]
    assert diff == [a for a in old.splitlines()
                    if not a.strip().startswith(("CGSolveQ(phys->qc", "CGSolve(grid", "ComputeQSource(phys->stmp",
                                                 "Corrector(phys->qc", "WPredictor(grid,phys"))]
    cc = ["gcc", "-fcommon", "-DNOMPI", "-DNONETCDF", "-w", f"-I{REF}", f"-I{ROOT}/include", "-c"]
    r = subprocess.run(cc + [str(phys), "-o", str(tmp_path / "phys.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(cc + [os.path.join(SHIM, "sgpu_suntans.c"), "-o", str(tmp_path / "shim.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", str(tmp_path / "shim.o")], capture_output=True, text=True).stdout
    for s_ in ("sgpu_ComputeQSource", "sgpu_Corrector", "sgpu_compute_qsource", "sgpu_corrector", "sgpu_step_grid"):
        assert s_ in syms


def test_patch_upred_mode_and_compile(tmp_path):
    """With "upred", the predictor's call in Solve moves to the adapter; the
    model's boundary functions stay where the reference calls them."""
    phys = tmp_path / "phys.c"
    shutil.copy(os.path.join(REF, "phys.c"), phys)
    r = subprocess.run(["sh", os.path.join(SHIM, "patch_phys.sh"), str(phys), "step", "upred"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    new = phys.read_text()
    assert new.count("sgpu_UPredictor(grid,phys,prop,myproc,numprocs,comm);") == 1
    old = open(os.path.join(REF, "phys.c")).read()
    diff = [a for a in new.splitlines() if "sgpu_" not in a]
    assert diff == [a for a in old.splitlines()
                    if not a.strip().startswith(("CGSolveQ(phys->qc", "CGSolve(grid", "ComputeQSource(phys->stmp",
                                                 "Corrector(phys->qc", "UPredictor(grid,phys", "WPredictor(grid,phys"))]
    cc = ["gcc", "-fcommon", "-DNOMPI", "-DNONETCDF", "-w", f"-I{REF}", f"-I{ROOT}/include", "-c"]
    r = subprocess.run(cc + [str(phys), "-o", str(tmp_path / "phys.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(cc + [os.path.join(SHIM, "sgpu_suntans.c"), "-o", str(tmp_path / "shim.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", str(tmp_path / "shim.o")], capture_output=True, text=True).stdout
    for s in ("sgpu_UPredictor", "sgpu_upredictor_vertical", "sgpu_upredictor_rhs", "sgpu_upredictor_finish",
              "BoundaryVelocities", "OpenBoundaryFluxes"):
        assert s in syms


def test_patch_fused_mode_and_compile(tmp_path):
    """With "fused", WPredictor's call becomes the one-call nonhydrostatic step
    and the three calls after it are commented out; nothing else changes."""
    phys = tmp_path / "phys.c"
    shutil.copy(os.path.join(REF, "phys.c"), phys)
    r = subprocess.run(["sh", os.path.join(SHIM, "patch_phys.sh"), str(phys), "fused", "upred"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    new = phys.read_text()
    assert new.count("sgpu_NonhydrostaticStep(grid,phys,prop,myproc,numprocs,comm);") == 1
    assert new.count("in sgpu_NonhydrostaticStep */") == 3
    lines = new.splitlines()
    i = next(n for n, a in enumerate(lines) if "sgpu_NonhydrostaticStep(grid,phys" in a)
    assert "ComputeQSource: in" in "\n".join(lines[i:i + 6])
    old = open(os.path.join(REF, "phys.c")).read()
    diff = [a for a in new.splitlines() if "sgpu_" not in a]
    assert diff == [a for a in old.splitlines()
                    if not a.strip().startswith(("CGSolveQ(phys->qc", "CGSolve(grid", "ComputeQSource(phys->stmp",
                                                 "Corrector(phys->qc", "UPredictor(grid,phys", "WPredictor(grid,phys"))]
    cc = ["gcc", "-fcommon", "-DNOMPI", "-DNONETCDF", "-w", f"-I{REF}", f"-I{ROOT}/include", "-c"]
    r = subprocess.run(cc + [str(phys), "-o", str(tmp_path / "phys.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(cc + [os.path.join(SHIM, "sgpu_suntans.c"), "-o", str(tmp_path / "shim.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", str(tmp_path / "shim.o")], capture_output=True, text=True).stdout
    for s in ("sgpu_NonhydrostaticStep", "sgpu_nonhydrostatic_step", "sgpu_WPredictor"):
        assert s in syms
    bad = subprocess.run(["sh", os.path.join(SHIM, "patch_phys.sh"), str(phys) + ".orig", "step", "fused"],
                         capture_output=True, text=True)
    assert bad.returncode == 2
