/*
 * sgpu_suntans.c -- drop-in adapter compiled INSIDE a SUNTANS source tree.
 *
 * Provides sgpu_CGSolveQ and sgpu_CGSolve with exactly the parameter lists of
 * the reference's static CGSolveQ (main/phys.c:50-52, defined 2411) and
 * CGSolve (main/phys.c:45-46, defined 3086).  patch_phys.sh redirects the two
 * call sites (main/phys.c:1280 in Solve and main/phys.c:2989 in UPredictor) to
 * them; nothing else in the model changes.  The adapter reads gridT / physT /
 * propT through the model's own headers and calls the C ABI of
 * include/suntans_gb300.h with the model's jagged arrays, so there is no
 * packing copy in the model.
 *
 * Behaviour kept from the reference:
 *   - the solution goes to q (phys->qc) and phys->h in place;
 *   - the same convergence messages at VERBOSE > 2 (phys.c:2527-2536,
 *     3204-3213);
 *   - a run with more than one process is refused (one GPU, one partition).
 * Differences: src/htmp and the scratch fields are left untouched (no caller
 * reads them after the solve); a solver failure prints the library's message
 * and returns instead of continuing silently.  There is no CPU fallback: a
 * missing GPU stops the run with an error.
 */
#include <stdio.h>
#include <stdlib.h>

#include "boundaries.h"
#include "grid.h"
#include "phys.h"
#include "suntans_gb300.h"

static sgpu_context *g_ctx = NULL;
static gridT *g_ctx_grid = NULL;

static void sgpu_die(const char *what, int rc) {
  fprintf(stderr, "sgpu: %s failed: %s (%s)\n", what, sgpu_status_string(rc),
          g_ctx ? sgpu_last_error(g_ctx) : "");
  exit(EXIT_FAILURE);
}

static void sgpu_ensure_context(gridT *grid, int numprocs) {
  sgpu_grid_desc d;
  int rc;
  if (numprocs > 1) {
    fprintf(stderr, "sgpu: the GPU solvers run one partition; start SUNTANS with one process\n");
    exit(EXIT_FAILURE);
  }
  if (g_ctx && g_ctx_grid == grid) return;
  if (g_ctx) sgpu_destroy(g_ctx);
  d.Nc = grid->Nc;
  d.Ne = grid->Ne;
  d.maxfaces = grid->maxfaces;
  d.Nkmax = grid->Nkmax;
  d.nfaces = grid->nfaces;
  d.neigh = grid->neigh;
  d.face = grid->face;
  d.Nk = grid->Nk;
  d.Nke = grid->Nke;
  d.cellp = grid->cellp;
  d.celldist = grid->celldist;
  d.Ac = grid->Ac;
  d.df = grid->df;
  d.dg = grid->dg;
  rc = sgpu_create(&d, 0, &g_ctx);
  if (rc != SGPU_OK) sgpu_die("sgpu_create", rc);
  g_ctx_grid = grid;
}

static void sgpu_props_from(const propT *prop, sgpu_props *p) {
  p->qprecond = prop->qprecond;
  p->qmaxiters = prop->qmaxiters;
  p->qepsilon = prop->qepsilon;
  p->hprecond = prop->hprecond;
  p->maxiters = prop->maxiters;
  p->epsilon = prop->epsilon;
  p->resnorm = prop->resnorm;
  p->grav = prop->grav;
  p->theta = prop->theta;
  p->dt = prop->dt;
}

void sgpu_CGSolveQ(REAL **q, REAL **src, REAL **c, gridT *grid, physT *phys, propT *prop, int myproc,
                   int numprocs, MPI_Comm comm) {
  sgpu_props p;
  sgpu_stats st;
  int rc;
  (void)comm;
  sgpu_ensure_context(grid, numprocs);
  sgpu_props_from(prop, &p);
  rc = sgpu_cgsolveq(g_ctx, grid->ctop, (const double *const *)grid->dzz, (const double *const *)grid->dzf,
                     phys->D, q, (const double *const *)src, (const double *const *)c, &p, &st);
  if (rc != SGPU_OK && rc != SGPU_MAXITER && rc != SGPU_BREAKDOWN) sgpu_die("sgpu_cgsolveq", rc);
  if (myproc == 0 && VERBOSE > 2) {
    double res = st.eps0 != 0 ? sqrt(st.eps / st.eps0) : 0;
    if (rc == SGPU_BREAKDOWN)
      printf("Warning... Time step %d, Pressure iteration broke down after %d steps (non-finite step)\n", prop->n,
             st.niters);
    else if (st.eps == 0)
      printf("Warning...Time step %d, norm of pressure source is 0.\n", prop->n);
    else if (rc == SGPU_MAXITER)
      printf("Warning... Time step %d, Pressure iteration not converging after %d steps! RES=%e > %.2e\n",
             prop->n, st.niters, res, prop->qepsilon);
    else
      printf("Time step %d, CGSolve pressure converged after %d iterations, res=%e < %.2e\n", prop->n,
             st.niters, res, prop->qepsilon);
  }
}

void sgpu_CGSolve(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  sgpu_props p;
  sgpu_stats st;
  int rc;
  (void)comm;
  sgpu_ensure_context(grid, numprocs);
  sgpu_props_from(prop, &p);
  rc = sgpu_cgsolve(g_ctx, phys->D, phys->h, phys->htmp, &p, &st);
  if (rc != SGPU_OK && rc != SGPU_MAXITER && rc != SGPU_BREAKDOWN) sgpu_die("sgpu_cgsolve", rc);
  if (myproc == 0 && VERBOSE > 2) {
    double res = st.eps0 != 0 ? sqrt(st.eps / st.eps0) : 0;
    if (rc == SGPU_BREAKDOWN)
      printf("Warning... Time step %d, Free-surface iteration broke down after %d steps (non-finite step)\n",
             prop->n, st.niters);
    else if (st.eps == 0)
      printf("Warning...Time step %d, norm of free-surface source is 0.\n", prop->n);
    else if (rc == SGPU_MAXITER)
      printf("Warning... Time step %d, Free-surface iteration not converging after %d steps! RES=%e > %.2e\n",
             prop->n, st.niters, res, prop->qepsilon);
    else
      printf("Time step %d, CGSolve free-surface converged after %d iterations, res=%e < %.2e\n", prop->n,
             st.niters, res, prop->epsilon);
  }
}

/* The steps on either side of CGSolveQ in Solve (main/phys.c:1273-1287), with
 * the reference's parameter lists: ComputeQSource (declared phys.c:53-54,
 * defined 2345) and Corrector (declared phys.c:55-56, defined 2301).  The
 * edge and normal fields they need beyond the solver's grid are uploaded once
 * per grid.  Same bits as the reference. */
static gridT *g_step_grid = NULL;

static void sgpu_ensure_step(gridT *grid, int numprocs) {
  int rc;
  sgpu_ensure_context(grid, numprocs);
  if (g_step_grid == grid) return;
  rc = sgpu_step_grid(g_ctx, grid->normal, grid->grad, grid->edgep, grid->edgedist);
  if (rc != SGPU_OK) sgpu_die("sgpu_step_grid", rc);
  g_step_grid = grid;
}

void sgpu_ComputeQSource(REAL **src, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs) {
  int rc;
  (void)myproc;
  sgpu_ensure_step(grid, numprocs);
  rc = sgpu_compute_qsource(g_ctx, grid->ctop, (const double *const *)grid->dzf, (const double *const *)phys->u,
                            (const double *const *)phys->utmp2, (const double *const *)phys->w,
                            (const double *const *)phys->wtmp2, prop->theta, prop->dt, src, phys->D);
  if (rc != SGPU_OK) sgpu_die("sgpu_compute_qsource", rc);
}

void sgpu_Corrector(REAL **qc, gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  int rc;
  (void)myproc;
  (void)comm;
  sgpu_ensure_step(grid, numprocs);
  rc = sgpu_corrector(g_ctx, grid->ctop, grid->etop, (const double *const *)grid->dzz, (const double *const *)qc,
                      phys->D, prop->dt, phys->u, phys->w, phys->q);
  if (rc != SGPU_OK) sgpu_die("sgpu_corrector", rc);
}

/* UPredictor (declared static at main/phys.c:39-40, defined 2579, called from
 * Solve at 1170) with the reference's parameter list.  The vertical predictor
 * (U***, E, D), the free-surface right-hand side, CGSolve and the steps after
 * it run on the device; the model's own BoundaryVelocities and
 * OpenBoundaryFluxes run on the host between them, where the reference calls
 * them, because they read the case's boundary data.  Needs cgsolver 1 and a
 * nonlinear free surface (linearFS 0).  Same bits as the reference apart from
 * CGSolve's parity bound. */
static gridT *g_up_grid = NULL;

void sgpu_UPredictor(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  sgpu_upred_fields f;
  sgpu_props p;
  sgpu_vgrid v;
  int rc, i, j, jptr, k;
  sgpu_ensure_step(grid, numprocs);
  if (prop->cgsolver != 1 || prop->linearFS) {
    fprintf(stderr, "sgpu: UPredictor on the GPU needs cgsolver 1 and linearFS 0\n");
    exit(EXIT_FAILURE);
  }
  if (g_up_grid != grid) {
    rc = sgpu_upredictor_grid(g_ctx, grid->edgep, grid->edgedist, grid->mark, grid->n1, grid->n2, grid->face,
                              grid->normal);
    if (rc != SGPU_OK) sgpu_die("sgpu_upredictor_grid", rc);
    g_up_grid = grid;
  }
  for (i = 0; i < grid->Nc; i++) /* 2595-2598 */
    for (k = 0; k < grid->Nk[i] + 1; k++) phys->wtmp2[i][k] = phys->w[i][k];
  for (j = 0; j < grid->Ne; j++) /* 2600-2604 */
    for (k = 0; k < grid->Nke[j]; k++) phys->utmp2[j][k] = phys->u[j][k];
  for (jptr = grid->edgedist[2]; jptr < grid->edgedist[3]; jptr++) { /* 2611-2618 */
    j = grid->edgep[jptr];
    for (k = grid->etop[j]; k < grid->Nke[j]; k++) phys->utmp[j][k] = phys->u[j][k];
  }
  f.u = (const double *const *)phys->u;
  f.w = (const double *const *)phys->w;
  f.nu_tv = (const double *const *)phys->nu_tv;
  f.nu_lax = (const double *const *)phys->nu_lax;
  f.tau_T = phys->tau_T;
  f.CdT = phys->CdT;
  f.CdB = phys->CdB;
  f.nu = prop->nu;
  f.laxWendroff_Vertical = prop->laxWendroff_Vertical;
  f.thetaM = prop->thetaM;
  f.nonlinear = prop->nonlinear;
  sgpu_props_from(prop, &p);
  rc = sgpu_upredictor_vertical(g_ctx, grid->ctop, grid->etop, (const double *const *)grid->dzz,
                                (const double *const *)grid->dzf, phys->h, &f, &p, phys->utmp, phys->ut, phys->D);
  if (rc == SGPU_BREAKDOWN) {
    printf("Error in function Predictor (U***=nan): %s\n", sgpu_last_error(g_ctx));
    exit(EXIT_FAILURE);
  }
  if (rc != SGPU_OK) sgpu_die("sgpu_upredictor_vertical", rc);
  BoundaryVelocities(grid, phys, prop, myproc, comm); /* 2961-2962 */
  OpenBoundaryFluxes(NULL, phys->utmp, NULL, grid, phys, prop);
  rc = sgpu_upredictor_rhs(g_ctx, grid->etop, (const double *const *)grid->dzf, (const double *const *)phys->u,
                           (const double *const *)phys->utmp, phys->h, &p, phys->htmp);
  if (rc != SGPU_OK) sgpu_die("sgpu_upredictor_rhs", rc);
  sgpu_CGSolve(grid, phys, prop, myproc, numprocs, comm);
  /* UpdateDZ's first block (option 0, 826-839): the old vertical grid */
  for (j = 0; j < grid->Ne; j++) grid->etopold[j] = grid->etop[j];
  for (i = 0; i < grid->Nc; i++) {
    grid->ctopold[i] = grid->ctop[i];
    for (k = 0; k < grid->ctop[i]; k++) grid->dzzold[i][k] = 0;
    for (k = grid->ctop[i]; k < grid->Nk[i]; k++) grid->dzzold[i][k] = grid->dzz[i][k];
  }
  v.dz = grid->dz;
  v.dv = grid->dv;
  v.dzbot = grid->dzbot;
  v.Nkc = grid->Nkc;
  v.smoothbot = grid->smoothbot;
  v.dzsmall = grid->dzsmall;
  rc = sgpu_upredictor_finish(g_ctx, &v, &p, grid->ctop, grid->etop, grid->dzz, (const double *const *)phys->utmp,
                              (const double *const *)phys->ut, phys->h, phys->active, phys->u);
  if (rc != SGPU_OK) sgpu_die("sgpu_upredictor_finish", rc);
  for (i = 0; i < grid->Nc; i++) /* 2993-3002 */
    if (!phys->active[i])
      phys->s[i][grid->Nk[i] - 1] = 0;
    else
      phys->hcorr[i] = 0;
}

/* WPredictor (declared static at main/phys.c:81-82, defined 2025, called from
 * Solve at 1271) with the reference's parameter list, for nonlinear 0 or 1,
 * conserveMomentum 0 and grids without type-2 or type-4 edges.  Its scratch
 * fields (phys->wtmp, stmp, wc, ut) are left untouched; nothing reads them
 * after it.  Same bits as the reference. */
static void sgpu_wpred_from(gridT *grid, physT *phys, propT *prop, sgpu_wpred_fields *f) {
  if ((prop->nonlinear != 0 && prop->nonlinear != 1) || prop->conserveMomentum ||
      grid->edgedist[3] > grid->edgedist[2] || grid->edgedist[5] > grid->edgedist[4]) {
    fprintf(stderr, "sgpu: WPredictor on the GPU needs nonlinear 0 or 1, conserveMomentum 0 and no type-2/4 edges\n");
    exit(EXIT_FAILURE);
  }
  f->q = (const double *const *)phys->q;
  f->nu_tv = (const double *const *)phys->nu_tv;
  f->nu_lax = (const double *const *)phys->nu_lax;
  f->utmp2 = (const double *const *)phys->utmp2;
  f->nu = prop->nu;
  f->nu_H = prop->nu_H;
  f->CdW = prop->CdW;
  f->laxWendroff_Vertical = prop->laxWendroff_Vertical;
  f->nonlinear = prop->nonlinear;
  f->conserveMomentum = prop->conserveMomentum;
  f->n = prop->n;
  f->AB = prop->AB;
}

void sgpu_WPredictor(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  sgpu_wpred_fields f;
  sgpu_props p;
  int rc;
  (void)myproc;
  (void)comm;
  sgpu_ensure_step(grid, numprocs);
  sgpu_wpred_from(grid, phys, prop, &f);
  sgpu_props_from(prop, &p);
  rc = sgpu_wpredictor(g_ctx, grid->ctop, (const double *const *)grid->dzz, &f, &p, phys->w, phys->Cn_W,
                       phys->Cn_W2);
  if (rc != SGPU_OK) sgpu_die("sgpu_wpredictor", rc);
}

/* The nonhydrostatic block of Solve (main/phys.c:1271-1289) in one call:
 * WPredictor -> ComputeQSource -> CGSolveQ -> Corrector with w, q, the
 * right-hand side, D and the correction kept on the device between them.
 * Same settings as sgpu_WPredictor; phys->stmp (the right-hand side) and
 * phys->D are not written back, because nothing in Solve reads them before
 * UPredictor forms them again. */
void sgpu_NonhydrostaticStep(gridT *grid, physT *phys, propT *prop, int myproc, int numprocs, MPI_Comm comm) {
  sgpu_wpred_fields f;
  sgpu_props p;
  sgpu_stats st;
  int rc;
  (void)comm;
  sgpu_ensure_step(grid, numprocs);
  sgpu_wpred_from(grid, phys, prop, &f);
  sgpu_props_from(prop, &p);
  rc = sgpu_nonhydrostatic_step(g_ctx, grid->ctop, grid->etop, (const double *const *)grid->dzz,
                                (const double *const *)grid->dzf, (const double *const *)phys->utmp2,
                                (const double *const *)phys->wtmp2, &f, phys->u, phys->w, phys->q, phys->qc,
                                (const double *const *)phys->stmp3, phys->Cn_W, phys->Cn_W2, &p, &st);
  if (rc != SGPU_OK && rc != SGPU_MAXITER && rc != SGPU_BREAKDOWN) sgpu_die("sgpu_nonhydrostatic_step", rc);
  if (myproc == 0 && VERBOSE > 2) {
    double res = st.eps0 != 0 ? sqrt(st.eps / st.eps0) : 0;
    if (rc == SGPU_BREAKDOWN)
      printf("Warning... Time step %d, Pressure iteration broke down after %d steps (non-finite step)\n", prop->n,
             st.niters);
    else if (st.eps == 0)
      printf("Warning...Time step %d, norm of pressure source is 0.\n", prop->n);
    else if (rc == SGPU_MAXITER)
      printf("Warning... Time step %d, Pressure iteration not converging after %d steps! RES=%e > %.2e\n",
             prop->n, st.niters, res, prop->qepsilon);
    else
      printf("Time step %d, CGSolve pressure converged after %d iterations, res=%e < %.2e\n", prop->n,
             st.niters, res, prop->qepsilon);
  }
}
