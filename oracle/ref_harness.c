/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Calls the reference's own static CGSolveQ / CGSolve and their helpers by
 * compiling the reference's main/phys.c into this translation unit (the
 * functions are static, main/phys.c:45-52, so they cannot be linked to from
 * outside).  The include path points at the reference sources where they lie;
 * nothing is copied.  Built by oracle/Makefile into oracle/_ref/ only where the
 * reference tree is present.
 *
 * The harness builds gridT / physT / propT whose jagged REAL** rows point into
 * the caller's flat arrays (layout in cg_oracle.h), so the solvers read and
 * write the caller's buffers in place, exactly as they do phys->qc and
 * phys->stmp in the model.
 *
 * Iteration counts: CGSolveQ / CGSolve return nothing.  Each solver iteration
 * calls the halo exchange on p exactly once (main/phys.c:2480, 3163), and the
 * prologue/epilogue call it a fixed number of times, so the harness counts
 * calls through -Wl,--wrap of ISendRecvCellData3D/2D.  With one partition the
 * exchange is a no-op (main/sendrecv.c:134-217 with Nneighs=0).
 */
#include "phys.c"
#include "gridio.h"
#include "cg_oracle.h"

static int g_calls3d, g_calls2d;
void __real_ISendRecvCellData3D(REAL **celldata, gridT *grid, int myproc, MPI_Comm comm);
void __real_ISendRecvCellData2D(REAL *celldata, gridT *grid, int myproc, MPI_Comm comm);
void __wrap_ISendRecvCellData3D(REAL **celldata, gridT *grid, int myproc, MPI_Comm comm) {
  g_calls3d++;
  __real_ISendRecvCellData3D(celldata, grid, myproc, comm);
}
void __wrap_ISendRecvCellData2D(REAL *celldata, gridT *grid, int myproc, MPI_Comm comm) {
  g_calls2d++;
  __real_ISendRecvCellData2D(celldata, grid, myproc, comm);
}

typedef struct {
  gridT grid;
  physT phys;
  propT prop;
  long *coff, *eoff;
  REAL **rows_free[64];
  int nrows_free;
  void *blk_free[96];
  int nblk_free;
} harness_t;

static REAL **jag_view(harness_t *H, const double *flat, const long *off, int n) {
  int i;
  REAL **rows = (REAL **)malloc(sizeof(REAL *) * (n > 0 ? n : 1));
  for (i = 0; i < n; i++) rows[i] = (REAL *)(flat + off[i]);
  H->rows_free[H->nrows_free++] = rows;
  return rows;
}
static REAL **jag_new(harness_t *H, int n, const int *len, int extra) {
  long tot = 0;
  int i;
  double *blk;
  for (i = 0; i < n; i++) tot += len[i] + extra;
  blk = (double *)calloc(tot + 1, sizeof(double));
  H->blk_free[H->nblk_free++] = blk;
  REAL **rows = (REAL **)malloc(sizeof(REAL *) * (n > 0 ? n : 1));
  tot = 0;
  for (i = 0; i < n; i++) { rows[i] = blk + tot; tot += len[i] + extra; }
  H->rows_free[H->nrows_free++] = rows;
  return rows;
}
static void *blk_new(harness_t *H, size_t bytes) {
  void *p = calloc(1, bytes + 16);
  H->blk_free[H->nblk_free++] = p;
  return p;
}

static void harness_init(harness_t *H, const sgo_grid *g, const double *D, const sgo_prop *pr) {
  int i, nf;
  memset(H, 0, sizeof(*H));
  H->coff = (long *)malloc(sizeof(long) * (g->Nc + 1));
  H->eoff = (long *)malloc(sizeof(long) * (g->Ne + 1));
  H->coff[0] = 0;
  for (i = 0; i < g->Nc; i++) H->coff[i + 1] = H->coff[i] + g->Nk[i];
  H->eoff[0] = 0;
  for (i = 0; i < g->Ne; i++) H->eoff[i + 1] = H->eoff[i] + g->Nke[i];

  gridT *G = &H->grid;
  G->Nc = g->Nc;
  G->Ne = g->Ne;
  G->maxfaces = g->maxfaces;
  G->Nkmax = g->Nkmax;
  G->nfaces = (int *)g->nfaces;
  G->neigh = (int *)g->neigh;
  G->face = (int *)g->face;
  G->Nk = (int *)g->Nk;
  G->Nke = (int *)g->Nke;
  G->ctop = (int *)g->ctop;
  G->cellp = (int *)g->cellp;
  G->celldist = (int *)g->celldist;
  G->Ac = (REAL *)g->Ac;
  G->df = (REAL *)g->df;
  G->dg = (REAL *)g->dg;
  G->Nneighs = 0;
  if (g->dzz) G->dzz = jag_view(H, g->dzz, H->coff, g->Nc);
  if (g->dzf) G->dzf = jag_view(H, g->dzf, H->eoff, g->Ne);

  physT *P = &H->phys;
  P->D = (REAL *)D;
  P->stmp2 = jag_new(H, g->Nc, g->Nk, 0);
  P->stmp3 = jag_new(H, g->Nc, g->Nk, 0);
  P->uold = jag_new(H, g->Nc, g->Nk, 0);
  P->wtmp = jag_new(H, g->Nc, g->Nk, 1);
  {
    int *qlen = (int *)malloc(sizeof(int) * g->maxfaces * g->Nc + 1);
    for (i = 0; i < g->Nc; i++)
      for (nf = 0; nf < g->maxfaces; nf++) qlen[i * g->maxfaces + nf] = g->Nk[i];
    P->qtmp = jag_new(H, g->maxfaces * g->Nc, qlen, 0);
    free(qlen);
  }
  P->a = (REAL *)blk_new(H, sizeof(REAL) * (g->Nkmax + 1));
  P->b = (REAL *)blk_new(H, sizeof(REAL) * (g->Nkmax + 1));
  P->c = (REAL *)blk_new(H, sizeof(REAL) * (g->Nkmax + 1));
  P->d = (REAL *)blk_new(H, sizeof(REAL) * (g->Nkmax + 1));
  P->hold = (REAL *)blk_new(H, sizeof(REAL) * g->Nc);
  P->htmp2 = (REAL *)blk_new(H, sizeof(REAL) * g->Nc);
  P->htmp3 = (REAL *)blk_new(H, sizeof(REAL) * g->Nc);
  P->hcoef = (REAL *)blk_new(H, sizeof(REAL) * g->Nc);
  P->hfcoef = (REAL *)blk_new(H, sizeof(REAL) * g->maxfaces * g->Nc);

  propT *Q = &H->prop;
  if (pr) {
    Q->qprecond = pr->qprecond;
    Q->qmaxiters = pr->qmaxiters;
    Q->qepsilon = pr->qepsilon;
    Q->hprecond = pr->hprecond;
    Q->maxiters = pr->maxiters;
    Q->epsilon = pr->epsilon;
    Q->resnorm = pr->resnorm;
    Q->grav = pr->grav;
    Q->theta = pr->theta;
    Q->dt = pr->dt;
  }
  VERBOSE = 0;
  WARNING = 0;
}

static void harness_free(harness_t *H) {
  int i;
  for (i = 0; i < H->nrows_free; i++) free(H->rows_free[i]);
  for (i = 0; i < H->nblk_free; i++) free(H->blk_free[i]);
  free(H->coff);
  free(H->eoff);
}

/* copy a harness jagged array (row length Nk[i]) out to a flat ragged array */
static void jag_out(const harness_t *H, const sgo_grid *g, REAL **src, double *dst) {
  int i;
  for (i = 0; i < g->Nc; i++) memcpy(dst + H->coff[i], src[i], sizeof(double) * g->Nk[i]);
}

void ref_cgsolveq(const sgo_grid *g, const double *D, double *q, double *src, double *c, const sgo_prop *pr,
                  sgo_result *res) {
  harness_t H;
  harness_init(&H, g, D, pr);
  REAL **Q = jag_view(&H, q, H.coff, g->Nc);
  REAL **S = jag_view(&H, src, H.coff, g->Nc);
  REAL **C = jag_view(&H, c, H.coff, g->Nc);
  g_calls3d = 0;
  CGSolveQ(Q, S, C, &H.grid, &H.phys, &H.prop, 0, 1, 0);
  if (res) {
    /* x before, p per iteration, x after; ConditionQ adds one for qprecond=1 */
    res->niters = g_calls3d - 2 - (pr->qprecond == 1 ? 1 : 0);
    res->eps = -1;
    res->eps0 = -1;
    res->t_setup = -1;
    res->t_loop = -1;
  }
  harness_free(&H);
}

void ref_cgsolve(const sgo_grid *g, const double *D, double *h, double *htmp, const sgo_prop *pr,
                 sgo_result *res) {
  harness_t H;
  harness_init(&H, g, D, pr);
  H.phys.h = h;
  H.phys.htmp = htmp;
  g_calls2d = 0;
  CGSolve(&H.grid, &H.phys, &H.prop, 0, 1, 0);
  if (res) {
    /* x for the lift, p per iteration, x at the end */
    res->niters = g_calls2d - 2;
    res->eps = -1;
    res->eps0 = -1;
    res->t_setup = -1;
    res->t_loop = -1;
  }
  harness_free(&H);
}

void ref_qcoefficients(const sgo_grid *g, const double *D, const double *c, int qprecond, double *coef,
                       double *fcoef) {
  harness_t H;
  sgo_prop pr;
  int i, nf;
  memset(&pr, 0, sizeof(pr));
  pr.qprecond = qprecond;
  harness_init(&H, g, D, &pr);
  REAL **C = jag_view(&H, c, H.coff, g->Nc);
  QCoefficients(H.phys.wtmp, H.phys.qtmp, C, &H.grid, &H.phys, &H.prop);
  jag_out(&H, g, H.phys.wtmp, coef);
  for (i = 0; i < g->Nc; i++)
    for (nf = 0; nf < g->maxfaces; nf++)
      memcpy(fcoef + (long)g->maxfaces * H.coff[i] + (long)nf * g->Nk[i], H.phys.qtmp[i * g->maxfaces + nf],
             sizeof(double) * g->Nk[i]);
  harness_free(&H);
}

void ref_operator_q(const sgo_grid *g, const double *D, const double *coef, const double *x, double *y) {
  harness_t H;
  harness_init(&H, g, D, NULL);
  REAL **CO = jag_view(&H, coef, H.coff, g->Nc);
  REAL **X = jag_view(&H, x, H.coff, g->Nc);
  REAL **Y = jag_view(&H, y, H.coff, g->Nc);
  OperatorQ(CO, X, Y, NULL, &H.grid, &H.phys, &H.prop);
  harness_free(&H);
}

void ref_operator_qc(const sgo_grid *g, const double *coef, const double *fcoef, const double *x, double *y) {
  harness_t H;
  int i, nf;
  harness_init(&H, g, NULL, NULL);
  REAL **CO = jag_view(&H, coef, H.coff, g->Nc);
  REAL **FC = (REAL **)malloc(sizeof(REAL *) * (g->maxfaces * g->Nc + 1));
  for (i = 0; i < g->Nc; i++)
    for (nf = 0; nf < g->maxfaces; nf++)
      FC[i * g->maxfaces + nf] = (REAL *)(fcoef + (long)g->maxfaces * H.coff[i] + (long)nf * g->Nk[i]);
  REAL **X = jag_view(&H, x, H.coff, g->Nc);
  REAL **Y = jag_view(&H, y, H.coff, g->Nc);
  OperatorQC(CO, FC, X, Y, NULL, &H.grid, &H.phys, &H.prop);
  free(FC);
  harness_free(&H);
}

void ref_condition_q(const sgo_grid *g, const double *D, double *c) {
  harness_t H;
  harness_init(&H, g, D, NULL);
  REAL **C = jag_view(&H, c, H.coff, g->Nc);
  ConditionQ(C, &H.grid, &H.phys, &H.prop, 0, 0);
  harness_free(&H);
}

void ref_preconditioner(const sgo_grid *g, const double *coef, const double *x, double *xc) {
  harness_t H;
  harness_init(&H, g, NULL, NULL);
  REAL **CO = jag_view(&H, coef, H.coff, g->Nc);
  REAL **X = jag_view(&H, x, H.coff, g->Nc);
  REAL **XC = jag_view(&H, xc, H.coff, g->Nc);
  Preconditioner(X, XC, CO, &H.grid, &H.phys, &H.prop);
  harness_free(&H);
}

void ref_hcoefficients(const sgo_grid *g, const double *D, const sgo_prop *p, double *hcoef, double *hfcoef) {
  harness_t H;
  harness_init(&H, g, D, p);
  HCoefficients(hcoef, hfcoef, &H.grid, &H.phys, &H.prop);
  harness_free(&H);
}

void ref_operator_h(const sgo_grid *g, const double *hcoef, const double *hfcoef, const double *x, double *y) {
  harness_t H;
  harness_init(&H, g, NULL, NULL);
  OperatorH((REAL *)x, y, (REAL *)hcoef, (REAL *)hfcoef, &H.grid, &H.phys, &H.prop);
  harness_free(&H);
}

/* the gridT fields of the steps around CGSolveQ, and a view of w-like rows
   (Nk[i]+1 levels per cell) */
static void harness_ext(harness_t *H, const sgo_grid *g, const sgo_ext *x) {
  H->grid.normal = (int *)x->normal;
  H->grid.grad = (int *)x->grad;
  H->grid.edgep = (int *)x->edgep;
  H->grid.edgedist = (int *)x->edgedist;
  H->grid.etop = (int *)x->etop;
}
static REAL **wrow_view(harness_t *H, const sgo_grid *g, const double *flat) {
  long *woff = (long *)blk_new(H, sizeof(long) * (g->Nc + 1));
  int i;
  woff[0] = 0;
  for (i = 0; i < g->Nc; i++) woff[i + 1] = woff[i] + g->Nk[i] + 1;
  return jag_view(H, flat, woff, g->Nc);
}

void ref_compute_qsource(const sgo_grid *g, const sgo_ext *x, const double *u, const double *utmp2,
                         const double *w, const double *wtmp2, const sgo_prop *p, double *src, double *D) {
  harness_t H;
  harness_init(&H, g, D, p);
  harness_ext(&H, g, x);
  H.phys.u = jag_view(&H, u, H.eoff, g->Ne);
  H.phys.utmp2 = jag_view(&H, utmp2, H.eoff, g->Ne);
  H.phys.w = wrow_view(&H, g, w);
  H.phys.wtmp2 = wrow_view(&H, g, wtmp2);
  REAL **S = jag_view(&H, src, H.coff, g->Nc);
  ComputeQSource(S, &H.grid, &H.phys, &H.prop, 0, 1);
  harness_free(&H);
}

void ref_corrector(const sgo_grid *g, const sgo_ext *x, const double *qc, const double *D,
                   const sgo_prop *p, double *u, double *w, double *q) {
  harness_t H;
  harness_init(&H, g, D, p);
  harness_ext(&H, g, x);
  H.phys.u = jag_view(&H, u, H.eoff, g->Ne);
  H.phys.w = wrow_view(&H, g, w);
  H.phys.q = jag_view(&H, q, H.coff, g->Nc);
  REAL **QC = jag_view(&H, qc, H.coff, g->Nc);
  Corrector(QC, &H.grid, &H.phys, &H.prop, 0, 1, 0);
  harness_free(&H);
}

static void harness_vgrid(harness_t *H, const sgo_vgrid *v) {
  H->grid.dz = (REAL *)v->dz;
  H->grid.dv = (REAL *)v->dv;
  H->grid.dzbot = (REAL *)v->dzbot;
  H->grid.Nkc = (int *)v->Nkc;
  H->grid.smoothbot = v->smoothbot;
  H->grid.dzsmall = v->dzsmall;
}

void ref_update_dz(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h, int linearFS,
                   int *ctop, int *etop, double *dzz, int *ctopold, int *etopold, double *dzzold) {
  harness_t H;
  sgo_prop pr;
  memset(&pr, 0, sizeof(pr));
  harness_init(&H, g, NULL, &pr);
  harness_ext(&H, g, x);
  harness_vgrid(&H, v);
  H.grid.ctop = ctop;
  H.grid.etop = etop;
  H.grid.ctopold = ctopold;
  H.grid.etopold = etopold;
  H.grid.dzz = jag_view(&H, dzz, H.coff, g->Nc);
  H.grid.dzzold = jag_view(&H, dzzold, H.coff, g->Nc);
  H.phys.h = (REAL *)h;
  H.prop.linearFS = linearFS;
  UpdateDZ(&H.grid, &H.phys, &H.prop, 0);
  harness_free(&H);
}

void ref_set_flux_height(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h,
                         const double *u, double *dzz, double *dzf) {
  harness_t H;
  long *foff;
  int j;
  sgo_prop pr;
  memset(&pr, 0, sizeof(pr));
  harness_init(&H, g, NULL, &pr);
  harness_ext(&H, g, x);
  harness_vgrid(&H, v);
  foff = (long *)blk_new(&H, sizeof(long) * (g->Ne + 1));
  foff[0] = 0;
  for (j = 0; j < g->Ne; j++) foff[j + 1] = foff[j] + v->Nkc[j];
  H.grid.dzz = jag_view(&H, dzz, H.coff, g->Nc);
  H.grid.dzf = jag_view(&H, dzf, foff, g->Ne);
  H.phys.h = (REAL *)h;
  H.phys.u = jag_view(&H, u, H.eoff, g->Ne);
  SetFluxHeight(&H.grid, &H.phys, &H.prop);
  harness_free(&H);
}

/* ---- formats: the reference's own run-time grid reader and field writers ----
 * ref_read_grid points DATADIR / DATAFILE at a folder holding a suntans.dat and
 * the grid files, and calls ReadGrid (main/gridio.c:54-187) for processor 0 of
 * 1; ref_grid_ints / ref_grid_dbls copy one named array of that gridT out.
 * Per-face arrays are copied whole (maxfaces per cell; slots past nfaces are
 * whatever ReadGrid left there).  Jagged nodal lists are copied flat. */
static gridT *g_rg;

int ref_read_grid(const char *dir, int *sizes) {
  snprintf(DATADIR, BUFFERLENGTH, "%s", dir);
  snprintf(DATAFILE, BUFFERLENGTH, "%s/suntans.dat", dir);
  VERBOSE = 0;
  g_rg = NULL;
  ReadGrid(&g_rg, 0, 1, 0);
  sizes[0] = g_rg->Nc;
  sizes[1] = g_rg->Ne;
  sizes[2] = g_rg->Np;
  sizes[3] = g_rg->maxfaces;
  sizes[4] = g_rg->Nkmax;
  sizes[5] = g_rg->Nneighs;
  return 0;
}

/* ref_read_main_grid: the grid step's own input reader on a folder holding a
 * suntans.dat (maxFaces and the points / edges / cells names) and the three
 * files: sizes from getsize, InitMainGrid (main/grid.c:337), ReadMainGrid
 * (main/gridio.c:256-266), as GetGrid (grid.c:110-135) runs them.  The arrays
 * are then read with ref_grid_ints / ref_grid_dbls. */
int ref_read_main_grid(const char *dir, int *sizes) {
  int Np, Ne, Nc;
  snprintf(DATADIR, BUFFERLENGTH, "%s", dir);
  snprintf(DATAFILE, BUFFERLENGTH, "%s/suntans.dat", dir);
  VERBOSE = 0;
  ReadGridFileNames(0);
  Np = MPI_GetSize(POINTSFILE, "ref_read_main_grid", 0);
  Ne = MPI_GetSize(EDGEFILE, "ref_read_main_grid", 0);
  Nc = MPI_GetSize(CELLSFILE, "ref_read_main_grid", 0);
  g_rg = NULL;
  InitMainGrid(&g_rg, Np, Ne, Nc, 0);
  ReadMainGrid(g_rg, 0);
  sizes[0] = g_rg->Nc;
  sizes[1] = g_rg->Ne;
  sizes[2] = g_rg->Np;
  sizes[3] = g_rg->maxfaces;
  sizes[4] = 0;
  sizes[5] = 0;
  return 0;
}

static long rg_flat_int(int **rows, const int *count, int n, int *out) {
  long p = 0;
  int i, k;
  for (i = 0; i < n; i++)
    for (k = 0; k < count[i]; k++) out[p++] = rows[i][k];
  return p;
}

long ref_grid_ints(const char *name, int *out) {
  gridT *G = g_rg;
  int n, Nc = G->Nc, Ne = G->Ne, Np = G->Np, mf = G->maxfaces;
#define RG_COPY(field, count)                                  \
  if (!strcmp(name, #field)) {                                 \
    memcpy(out, G->field, sizeof(int) * (size_t)(count));      \
    return (count);                                            \
  }
  RG_COPY(nfaces, Nc) RG_COPY(Nk, Nc) RG_COPY(mnptr, Nc) RG_COPY(cellp, Nc)
  RG_COPY(face, Nc * mf) RG_COPY(neigh, Nc * mf) RG_COPY(normal, Nc * mf) RG_COPY(cells, Nc * mf)
  RG_COPY(Nke, Ne) RG_COPY(Nkc, Ne) RG_COPY(mark, Ne) RG_COPY(edge_id, Ne) RG_COPY(eptr, Ne)
  RG_COPY(edgep, Ne) RG_COPY(grad, 2 * Ne) RG_COPY(gradf, 2 * Ne)
  RG_COPY(celldist, MAXBCTYPES - 1) RG_COPY(edgedist, MAXMARKS - 1)
  RG_COPY(localtoglobalpoints, Np) RG_COPY(numppneighs, Np) RG_COPY(numpeneighs, Np)
  RG_COPY(numpcneighs, Np) RG_COPY(Nkp, Np)
#undef RG_COPY
  if (!strcmp(name, "edges")) {
    for (n = 0; n < Ne; n++) {
      out[2 * n] = G->edges[NUMEDGECOLUMNS * n];
      out[2 * n + 1] = G->edges[NUMEDGECOLUMNS * n + 1];
    }
    return 2 * Ne;
  }
  if (!strcmp(name, "ppneighs")) return rg_flat_int(G->ppneighs, G->numppneighs, Np, out);
  if (!strcmp(name, "peneighs")) return rg_flat_int(G->peneighs, G->numpeneighs, Np, out);
  if (!strcmp(name, "pcneighs")) return rg_flat_int(G->pcneighs, G->numpcneighs, Np, out);
  return -1;
}

long ref_grid_dbls(const char *name, double *out) {
  gridT *G = g_rg;
  int i, k, Nc = G->Nc, Ne = G->Ne, Np = G->Np, mf = G->maxfaces;
  long p = 0;
#define RG_COPY(field, count)                                  \
  if (!strcmp(name, #field)) {                                 \
    memcpy(out, G->field, sizeof(double) * (size_t)(count));   \
    return (count);                                            \
  }
  RG_COPY(xv, Nc) RG_COPY(yv, Nc) RG_COPY(Ac, Nc) RG_COPY(dv, Nc) RG_COPY(def, Nc * mf)
  RG_COPY(df, Ne) RG_COPY(dg, Ne) RG_COPY(n1, Ne) RG_COPY(n2, Ne) RG_COPY(xe, Ne) RG_COPY(ye, Ne)
  RG_COPY(xp, Np) RG_COPY(yp, Np) RG_COPY(dz, G->Nkmax)
#undef RG_COPY
  if (!strcmp(name, "Actotal")) {
    for (i = 0; i < Np; i++)
      for (k = 0; k < G->Nkp[i]; k++) out[p++] = G->Actotal[i][k];
    return p;
  }
  return -1;
}

/* Write2DData / Write3DData (main/physio.c:29-105) without merging, on a gridT
 * that holds only what they read (Nc, Nkmax, Nk).  Rows of the 3-D field hold
 * Nk[i] + extra values laid end to end in flat. */
int ref_write_2d(const char *path, int Nc, const double *x) {
  gridT G;
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  memset(&G, 0, sizeof(G));
  G.Nc = Nc;
  Write2DData((REAL *)x, 0, f, "", &G, 1, 0, 0);
  fclose(f);
  return 0;
}

int ref_write_3d(const char *path, int Nc, int Nkmax, const int *Nk, const double *flat, int extra) {
  gridT G;
  long p = 0;
  int i;
  REAL **rows = (REAL **)malloc(sizeof(REAL *) * (Nc > 0 ? Nc : 1));
  REAL *tmp = (REAL *)malloc(sizeof(REAL) * (Nc > 0 ? Nc : 1));
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  for (i = 0; i < Nc; i++) {
    rows[i] = (REAL *)(flat + p);
    p += Nk[i] + extra;
  }
  memset(&G, 0, sizeof(G));
  G.Nc = Nc;
  G.Nkmax = Nkmax;
  G.Nk = (int *)Nk;
  Write3DData(rows, tmp, 0, f, "", &G, 1, 0, 0);
  fclose(f);
  free(rows);
  free(tmp);
  return 0;
}

/* The reference's UPredictor (main/phys.c:2579-3077) with cgsolver 1 and no
 * NetCDF boundary data.  Its scratch columns and physT fields are zeroed
 * allocations; boundary_u/v/w have one row of Nkmax per edge of marks 2-4. */
int ref_upredictor(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_upred *up,
                   const sgo_ubnd *b, const sgo_prop *p, double *u, double *h, double *utmp, double *E,
                   double *D, int *ctop, int *etop, double *dzz, unsigned char *active, sgo_result *res) {
  harness_t H;
  int nb = b->edgedist[5] - b->edgedist[2], i, *brow;
  harness_init(&H, g, D, p);
  harness_ext(&H, g, x);
  harness_vgrid(&H, v);
  H.grid.edgep = (int *)b->edgep;
  H.grid.edgedist = (int *)b->edgedist;
  H.grid.mark = (int *)b->mark;
  H.grid.n1 = (REAL *)b->n1;
  H.grid.n2 = (REAL *)b->n2;
  H.grid.ctop = ctop;
  H.grid.etop = etop;
  H.grid.ctopold = (int *)blk_new(&H, sizeof(int) * g->Nc);
  H.grid.etopold = (int *)blk_new(&H, sizeof(int) * g->Ne);
  H.grid.dzz = jag_view(&H, dzz, H.coff, g->Nc);
  H.grid.dzzold = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.a = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.b = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.c = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.d = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.ap = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.am = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.bp = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.bm = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.u = jag_view(&H, u, H.eoff, g->Ne);
  H.phys.utmp = jag_view(&H, utmp, H.eoff, g->Ne);
  H.phys.ut = jag_view(&H, E, H.eoff, g->Ne);
  H.phys.utmp2 = jag_new(&H, g->Ne, g->Nke, 0);
  H.phys.w = wrow_view(&H, g, up->w);
  H.phys.wtmp2 = jag_new(&H, g->Nc, g->Nk, 1);
  H.phys.h = h;
  H.phys.htmp = (REAL *)blk_new(&H, sizeof(REAL) * g->Nc);
  H.phys.hcorr = (REAL *)blk_new(&H, sizeof(REAL) * g->Nc);
  H.phys.active = active;
  H.phys.s = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.uc = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.vc = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.tau_T = (REAL *)up->tau_T;
  H.phys.CdT = (REAL *)up->CdT;
  H.phys.CdB = (REAL *)up->CdB;
  H.phys.nu_tv = jag_view(&H, up->nu_tv, H.coff, g->Nc);
  H.phys.nu_lax = jag_view(&H, up->nu_lax, H.coff, g->Nc);
  brow = (int *)malloc(sizeof(int) * (nb > 0 ? nb : 1));
  for (i = 0; i < nb; i++) brow[i] = g->Nkmax;
  H.phys.boundary_u = jag_new(&H, nb, brow, 0);
  H.phys.boundary_v = jag_new(&H, nb, brow, 0);
  H.phys.boundary_w = jag_new(&H, nb, brow, 0);
  free(brow);
  H.prop.nu = up->nu;
  H.prop.laxWendroff_Vertical = up->laxWendroff_Vertical;
  H.prop.thetaM = up->thetaM;
  H.prop.nonlinear = up->nonlinear;
  H.prop.cgsolver = 1;
  H.prop.netcdfBdy = 0;
  H.prop.thetaramptime = 0;
  H.prop.linearFS = 0;
  g_calls2d = 0;
  UPredictor(&H.grid, &H.phys, &H.prop, 0, 1, 0);
  if (res) {
    /* BoundaryVelocities exchanges h once, then as in ref_cgsolve */
    res->niters = g_calls2d - 3;
    res->eps = -1;
    res->eps0 = -1;
    res->t_setup = -1;
    res->t_loop = -1;
  }
  harness_free(&H);
  return 0;
}

/* The reference's WPredictor (main/phys.c:2025-2287).  Its edge loops read
 * edgedist[0..5]; the harness passes the computational edges with empty
 * ranges for marks 1-4.  phys->ut and utmp2 get rows of max(Nk) of the
 * edge's cells (the model's Nkc), zero past Nke, as the model allocates them;
 * Cn_W / Cn_W2 rows of Nk+1 are copied in and out of the caller's rows of Nk. */
int ref_wpredictor(const sgo_grid *g, const sgo_ext *x, const sgo_wpred *wp, const sgo_prop *p, double *w,
                   double *Cn_W, double *Cn_W2) {
  harness_t H;
  int i, j, k, ed[6], *nkc;
  REAL **cw, **cw2, **ut2;
  harness_init(&H, g, NULL, p);
  harness_ext(&H, g, x);
  ed[0] = x->edgedist[0];
  ed[1] = ed[2] = ed[3] = ed[4] = ed[5] = x->edgedist[1];
  H.grid.edgedist = ed;
  nkc = (int *)blk_new(&H, sizeof(int) * (g->Ne + 1));
  for (j = 0; j < g->Ne; j++) {
    int c0 = x->grad[2 * j], c1 = x->grad[2 * j + 1], m = 0;
    if (c0 >= 0 && g->Nk[c0] > m) m = g->Nk[c0];
    if (c1 >= 0 && g->Nk[c1] > m) m = g->Nk[c1];
    nkc[j] = m > g->Nke[j] ? m : g->Nke[j];
  }
  H.phys.a = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.b = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.c = (REAL *)blk_new(&H, sizeof(REAL) * (g->Nkmax + 2));
  H.phys.w = wrow_view(&H, g, w);
  H.phys.wtmp = jag_new(&H, g->Nc, g->Nk, 1);
  H.phys.stmp = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.wc = jag_new(&H, g->Nc, g->Nk, 0);
  H.phys.ut = jag_new(&H, g->Ne, nkc, 0);
  ut2 = jag_new(&H, g->Ne, nkc, 0);
  for (j = 0; j < g->Ne; j++)
    for (k = 0; k < g->Nke[j]; k++) ut2[j][k] = wp->utmp2[H.eoff[j] + k];
  H.phys.utmp2 = ut2;
  cw = jag_new(&H, g->Nc, g->Nk, 1);
  cw2 = jag_new(&H, g->Nc, g->Nk, 1);
  for (i = 0; i < g->Nc; i++)
    for (k = 0; k < g->Nk[i]; k++) {
      cw[i][k] = Cn_W[H.coff[i] + k];
      cw2[i][k] = Cn_W2[H.coff[i] + k];
    }
  H.phys.Cn_W = cw;
  H.phys.Cn_W2 = cw2;
  H.phys.q = jag_view(&H, wp->q, H.coff, g->Nc);
  H.phys.nu_tv = jag_view(&H, wp->nu_tv, H.coff, g->Nc);
  H.phys.nu_lax = jag_view(&H, wp->nu_lax, H.coff, g->Nc);
  H.phys.boundary_w = jag_new(&H, 1, g->Nk, 0);
  H.prop.n = wp->n;
  H.prop.AB = wp->AB;
  H.prop.nonlinear = wp->nonlinear;
  H.prop.conserveMomentum = wp->conserveMomentum;
  H.prop.nu = wp->nu;
  H.prop.nu_H = wp->nu_H;
  H.prop.CdW = wp->CdW;
  H.prop.laxWendroff_Vertical = wp->laxWendroff_Vertical;
  WPredictor(&H.grid, &H.phys, &H.prop, 0, 1, 0);
  for (i = 0; i < g->Nc; i++)
    for (k = 0; k < g->Nk[i]; k++) {
      Cn_W[H.coff[i] + k] = cw[i][k];
      Cn_W2[H.coff[i] + k] = cw2[i][k];
    }
  harness_free(&H);
  return 0;
}
