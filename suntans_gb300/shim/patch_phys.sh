#!/bin/sh
# Redirects the two elliptic solves of a SUNTANS main/phys.c to the GPU
# adapter (sgpu_suntans.c).  Usage:  sh patch_phys.sh path/to/main/phys.c [step] [upred]
# Edits in place and keeps phys.c.orig.  Exactly two call sites change:
#   Solve       main/phys.c:1280  CGSolveQ(phys->qc,phys->stmp,phys->stmp3,...)
#   UPredictor  main/phys.c:2989  CGSolve(grid,phys,prop,myproc,numprocs,comm)
# With "step", the nonhydrostatic steps around CGSolveQ in Solve move to the GPU too:
#   main/phys.c:1271  WPredictor(grid,phys,prop,myproc,numprocs,comm)
#   main/phys.c:1274  ComputeQSource(phys->stmp,...)
#   main/phys.c:1289  Corrector(phys->qc,...)
# With "fused" (instead of "step"), those four calls become one, the device
# keeping w, q, the right-hand side and the correction between them:
#   main/phys.c:1271  sgpu_NonhydrostaticStep(grid,phys,prop,myproc,numprocs,comm)
#   main/phys.c:1274, 1280, 1289  commented out
# With "upred", the whole predictor does (its call in Solve):
#   main/phys.c:1170  UPredictor(grid,phys,prop,myproc,numprocs,comm)
set -e
f="$1"
[ -f "$f" ] || { echo "usage: $0 main/phys.c [step|fused] [upred]" >&2; exit 2; }
step=0; upred=0; fused=0
for a in "$2" "$3"; do
  case "$a" in step) step=1 ;; fused) fused=1 ;; upred) upred=1 ;; "") ;; *) echo "unknown mode $a" >&2; exit 2 ;; esac
done
[ "$step" = 1 ] && [ "$fused" = 1 ] && { echo "patch_phys.sh: step and fused exclude each other" >&2; exit 2; }
cp "$f" "$f.orig"
sed -i \
  -e 's/^\([[:space:]]*\)CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);/\1sgpu_CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);/' \
  -e 's/^\([[:space:]]*\)CGSolve(grid,phys,prop,myproc,numprocs,comm);/\1sgpu_CGSolve(grid,phys,prop,myproc,numprocs,comm);/' \
  "$f"
# declarations, right after #include "phys.h"
sed -i '0,/^#include "phys.h"/s//#include "phys.h"\
void sgpu_CGSolveQ(REAL **q, REAL **src, REAL **c, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);\
void sgpu_CGSolve(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);/' "$f"
if [ "$upred" = 1 ]; then
  sed -i -e 's/^\([[:space:]]*\)UPredictor(grid,phys,prop,myproc,numprocs,comm);/\1sgpu_UPredictor(grid,phys,prop,myproc,numprocs,comm);/' "$f"
  sed -i '0,/^#include "phys.h"/s//#include "phys.h"\
void sgpu_UPredictor(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);/' "$f"
  m=$(grep -c 'sgpu_UPredictor' "$f")
  [ "$m" -ge 2 ] || { echo "patch_phys.sh: UPredictor call site not found ($m)" >&2; mv "$f.orig" "$f"; exit 1; }
fi
if [ "$step" = 1 ]; then
  sed -i \
    -e 's/^\([[:space:]]*\)ComputeQSource(phys->stmp,grid,phys,prop,myproc,numprocs);/\1sgpu_ComputeQSource(phys->stmp,grid,phys,prop,myproc,numprocs);/' \
    -e 's/^\([[:space:]]*\)Corrector(phys->qc,grid,phys,prop,myproc,numprocs,comm);/\1sgpu_Corrector(phys->qc,grid,phys,prop,myproc,numprocs,comm);/' \
    -e 's/^\([[:space:]]*\)WPredictor(grid,phys,prop,myproc,numprocs,comm);/\1sgpu_WPredictor(grid,phys,prop,myproc,numprocs,comm);/' \
    "$f"
  sed -i '0,/^#include "phys.h"/s//#include "phys.h"\
void sgpu_ComputeQSource(REAL **src, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs);\
void sgpu_Corrector(REAL **qc, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);\
void sgpu_WPredictor(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);/' "$f"
  m=$(grep -c 'sgpu_ComputeQSource\|sgpu_Corrector\|sgpu_WPredictor' "$f")
  [ "$m" -ge 6 ] || { echo "patch_phys.sh: step call sites not found ($m)" >&2; mv "$f.orig" "$f"; exit 1; }
fi
if [ "$fused" = 1 ]; then
  sed -i \
    -e 's/^\([[:space:]]*\)WPredictor(grid,phys,prop,myproc,numprocs,comm);/\1sgpu_NonhydrostaticStep(grid,phys,prop,myproc,numprocs,comm);/' \
    -e 's/^\([[:space:]]*\)ComputeQSource(phys->stmp,grid,phys,prop,myproc,numprocs);/\1\/* ComputeQSource: in sgpu_NonhydrostaticStep *\//' \
    -e 's/^\([[:space:]]*\)sgpu_CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);/\1\/* CGSolveQ: in sgpu_NonhydrostaticStep *\//' \
    -e 's/^\([[:space:]]*\)Corrector(phys->qc,grid,phys,prop,myproc,numprocs,comm);/\1\/* Corrector: in sgpu_NonhydrostaticStep *\//' \
    "$f"
  sed -i '0,/^#include "phys.h"/s//#include "phys.h"\
void sgpu_NonhydrostaticStep(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);/' "$f"
  m=$(grep -c 'in sgpu_NonhydrostaticStep\|sgpu_NonhydrostaticStep(grid,' "$f")
  [ "$m" -eq 4 ] || { echo "patch_phys.sh: nonhydrostatic call sites not found ($m)" >&2; mv "$f.orig" "$f"; exit 1; }
fi
n=$(grep -c 'sgpu_CGSolve' "$f")
[ "$n" -ge $((4 - fused)) ] || { echo "patch_phys.sh: expected call sites not found ($n)" >&2; mv "$f.orig" "$f"; exit 1; }
echo "patched $f ($n references)"
