#!/bin/sh
# Redirects the two elliptic solves of a SUNTANS main/phys.c to the GPU
# adapter (sgpu_suntans.c).  Usage:  sh patch_phys.sh path/to/main/phys.c
# Edits in place and keeps phys.c.orig.  Exactly two call sites change:
#   Solve       main/phys.c:1280  CGSolveQ(phys->qc,phys->stmp,phys->stmp3,...)
#   UPredictor  main/phys.c:2989  CGSolve(grid,phys,prop,myproc,numprocs,comm)
set -e
f="$1"
[ -f "$f" ] || { echo "usage: $0 main/phys.c" >&2; exit 2; }
cp "$f" "$f.orig"
sed -i \
  -e 's/^\([[:space:]]*\)CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);/\1sgpu_CGSolveQ(phys->qc,phys->stmp,phys->stmp3,grid,phys,prop,myproc,numprocs,comm);/' \
  -e 's/^\([[:space:]]*\)CGSolve(grid,phys,prop,myproc,numprocs,comm);/\1sgpu_CGSolve(grid,phys,prop,myproc,numprocs,comm);/' \
  "$f"
# declarations, right after #include "phys.h"
sed -i '0,/^#include "phys.h"/s//#include "phys.h"\
void sgpu_CGSolveQ(REAL **q, REAL **src, REAL **c, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);\
void sgpu_CGSolve(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm);/' "$f"
n=$(grep -c 'sgpu_CGSolve' "$f")
[ "$n" -ge 4 ] || { echo "patch_phys.sh: expected call sites not found ($n)" >&2; mv "$f.orig" "$f"; exit 1; }
echo "patched $f ($n references)"
