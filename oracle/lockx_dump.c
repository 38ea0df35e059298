/*
 * lockx_dump.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Records the inputs and outputs of every elliptic solve of a run of the
 * reference model itself.  It is compiled together with a copy of the
 * reference's main/phys.c whose two solver call sites were redirected by
 * suntans_gb300/shim/patch_phys.sh (Solve, main/phys.c:1280, and UPredictor,
 * main/phys.c:2989): the copy's sgpu_CGSolveQ / sgpu_CGSolve land here, write
 * what the solve reads, call the reference's own static CGSolveQ / CGSolve
 * (visible because the copy is #included into this file) and write what it
 * returns.  tests/golden/make_lockexchange_golden.py turns the record file
 * into fixtures.
 *
 * Two deviations from the reference at the call boundary, both the oracle's
 * documented fixes: CGSolveQ gets a preconditioner buffer c of its own (the
 * call site passes phys->stmp3, which is also CGSolveQ's residual, so with
 * qprecond 1 the final rescale divides by the converged residual), and qc, the
 * pressure-correction warm start that the reference never initialises
 * (main/phys.c:193, 260), is zeroed before the first solve.
 *
 * Record file "solver_dump.bin" in the working directory: a sequence of
 * arrays, each  char type ('i' int32, 'd' float64), int32 count, payload;
 * records are a tag array (int32: kind, step) followed by the kind's arrays
 * (see write_grid, sgpu_CGSolveQ, sgpu_CGSolve).
 */
#include "phys_patched.c"

static FILE *g_dump = NULL;
static int g_calls3 = 0, g_calls2 = 0;
static REAL **g_c = NULL;   /* CGSolveQ's own preconditioner buffer */
static int g_first_q = 1;

void __real_ISendRecvCellData3D(REAL **celldata, gridT *grid, int myproc, MPI_Comm comm);
void __real_ISendRecvCellData2D(REAL *celldata, gridT *grid, int myproc, MPI_Comm comm);
/* one halo exchange per solver iteration (plus a fixed number around it) */
void __wrap_ISendRecvCellData3D(REAL **celldata, gridT *grid, int myproc, MPI_Comm comm) {
  g_calls3++;
  __real_ISendRecvCellData3D(celldata, grid, myproc, comm);
}
void __wrap_ISendRecvCellData2D(REAL *celldata, gridT *grid, int myproc, MPI_Comm comm) {
  g_calls2++;
  __real_ISendRecvCellData2D(celldata, grid, myproc, comm);
}

static void wr(char t, const void *p, int n) {
  fwrite(&t, 1, 1, g_dump);
  fwrite(&n, sizeof(int), 1, g_dump);
  fwrite(p, t == 'i' ? sizeof(int) : sizeof(double), (size_t)n, g_dump);
}
static void wr_tag(int kind, int step) {
  int t[2] = {kind, step};
  wr('i', t, 2);
}
/* jagged rows laid end to end: row r has len[r] entries */
static void wr_jag(REAL **a, const int *len, int nrows) {
  int r, n = 0;
  double *flat;
  for (r = 0; r < nrows; r++) n += len[r];
  flat = (double *)malloc(sizeof(double) * (n + 1));
  n = 0;
  for (r = 0; r < nrows; r++) {
    memcpy(flat + n, a[r], sizeof(double) * len[r]);
    n += len[r];
  }
  wr('d', flat, n);
  free(flat);
}

/* kind 0: the grid (fields that do not change between steps) and the properties */
static void write_grid(gridT *g, propT *prop) {
  int sizes[4] = {g->Nc, g->Ne, g->maxfaces, g->Nkmax};
  double pr[10] = {prop->dt, prop->theta, GRAV, prop->epsilon, prop->qepsilon, prop->resnorm,
                   (double)prop->maxiters, (double)prop->qmaxiters, (double)prop->hprecond, (double)prop->qprecond};
  wr_tag(0, 0);
  wr('i', sizes, 4);
  wr('d', pr, 10);
  wr('i', g->nfaces, g->Nc);
  wr('i', g->neigh, g->Nc * g->maxfaces);
  wr('i', g->face, g->Nc * g->maxfaces);
  wr('i', g->Nk, g->Nc);
  wr('i', g->Nke, g->Ne);
  wr('i', g->cellp, g->Nc);
  wr('i', g->celldist, 3);
  wr('d', g->Ac, g->Nc);
  wr('d', g->df, g->Ne);
  wr('d', g->dg, g->Ne);
  wr('d', g->xv, g->Nc);
  wr('d', g->yv, g->Nc);
}

static void open_dump(gridT *grid, propT *prop) {
  if (g_dump) return;
  g_dump = fopen("solver_dump.bin", "wb");
  if (!g_dump) {
    printf("lockx_dump: cannot open solver_dump.bin\n");
    exit(1);
  }
  write_grid(grid, prop);
}

/* kind 1: CGSolveQ -- ctop, dzz, dzf, D, q (in), src (in); then q (out), iterations */
void sgpu_CGSolveQ(REAL **q, REAL **src, REAL **c, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs,
                   MPI_Comm comm) {
  int i, n;
  open_dump(grid, prop);
  if (!g_c) {
    g_c = (REAL **)malloc(sizeof(REAL *) * grid->Nc);
    for (i = 0; i < grid->Nc; i++) g_c[i] = (REAL *)calloc(grid->Nk[i] + 1, sizeof(REAL));
  }
  if (g_first_q) {
    for (i = 0; i < grid->Nc; i++) memset(q[i], 0, sizeof(REAL) * grid->Nk[i]);
    g_first_q = 0;
  }
  wr_tag(1, prop->n);
  wr('i', grid->ctop, grid->Nc);
  wr_jag(grid->dzz, grid->Nk, grid->Nc);
  wr_jag(grid->dzf, grid->Nke, grid->Ne);
  wr('d', phys->D, grid->Ne);
  wr_jag(q, grid->Nk, grid->Nc);
  wr_jag(src, grid->Nk, grid->Nc);
  g_calls3 = 0;
  CGSolveQ(q, src, g_c, grid, phys, prop, myproc, numprocs, comm);
  /* halo calls: x before the loop, p once per iteration, x after it, and one
     more inside ConditionQ for qprecond 1 */
  n = g_calls3 - 2 - (prop->qprecond == 1 ? 1 : 0);
  wr_jag(q, grid->Nk, grid->Nc);
  wr('i', &n, 1);
  fflush(g_dump);
}

/* kind 2: CGSolve -- D, h (in), htmp (in); then h (out), iterations */
void sgpu_CGSolve(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  int n;
  open_dump(grid, prop);
  wr_tag(2, prop->n);
  wr('d', phys->D, grid->Ne);
  wr('d', phys->h, grid->Nc);
  wr('d', phys->htmp, grid->Nc);
  g_calls2 = 0;
  CGSolve(grid, phys, prop, myproc, numprocs, comm);
  /* halo calls: x for the boundary lift, p once per iteration, x at the end */
  n = g_calls2 - 2;
  wr('d', phys->h, grid->Nc);
  wr('i', &n, 1);
  fflush(g_dump);
}
