/*
 * cg_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Flat-array description of a SUNTANS grid and the two elliptic solves, shared
 * by the two CPU oracles of this repository:
 *
 *   cg_oracle.c   a plain-C restatement of the reference algorithm (the "port"),
 *                 compiled on any host with -ffp-contract=off so that its
 *                 floating-point results are the same bits on x86 and Arm;
 *   ref_harness.c a thin wrapper that #includes the reference's own
 *                 main/phys.c and calls its static CGSolveQ / CGSolve
 *                 (built only where the reference sources are present).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
 * these functions, and only as the checker or the timed CPU baseline.  The
 * product (suntans_gb300/) never calls them.
 *
 * Ragged 3-D fields are flat arrays: cell i occupies [coff[i], coff[i]+Nk[i])
 * with coff the exclusive prefix sum of Nk over cell index i (natural cell
 * order, not cellp order); edge j of dzf occupies [eoff[j], eoff[j]+Nke[j]).
 * This is the reference's jagged REAL** (main/phys.c:247-282) laid end to end.
 */
#ifndef SUNTANS_CG_ORACLE_H
#define SUNTANS_CG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgo_grid {
  int Nc;              /* cells (computational + type-3 boundary), gridT.Nc      */
  int Ne;              /* edges, gridT.Ne                                         */
  int maxfaces;        /* gridT.maxfaces                                          */
  int Nkmax;           /* gridT.Nkmax                                             */
  const int *nfaces;   /* [Nc]                                                    */
  const int *neigh;    /* [Nc*maxfaces], -1 = no neighbour                        */
  const int *face;     /* [Nc*maxfaces], edge index                               */
  const int *Nk;       /* [Nc]                                                    */
  const int *Nke;      /* [Ne]                                                    */
  const int *ctop;     /* [Nc]                                                    */
  const int *cellp;    /* [celldist[2]]                                           */
  const int *celldist; /* [3]: computational [0,1), type-3 boundary [1,2)         */
  const double *Ac;    /* [Nc]                                                    */
  const double *df;    /* [Ne]                                                    */
  const double *dg;    /* [Ne]                                                    */
  const double *dzz;   /* ragged per cell, sum(Nk)                               */
  const double *dzf;   /* ragged per edge, sum(Nke)                              */
} sgo_grid;

typedef struct sgo_prop {
  int qprecond;        /* 0 none, 1 diagonal scaling, 2 column tridiagonal        */
  int qmaxiters;
  double qepsilon;
  int hprecond;        /* 0 none, 1 Jacobi                                        */
  int maxiters;
  double epsilon;
  double resnorm;      /* propT.resnorm is a REAL in the reference (phys.h:185)  */
  double grav, theta, dt;
} sgo_prop;

typedef struct sgo_result {
  int niters;          /* solver iterations executed (operator applications in   
                          the loop; the reference's n, plus one when it broke)   */
  double eps, eps0;    /* last eps and the normaliser eps0                        */
} sgo_result;

/* The gridT fields the steps on either side of CGSolveQ read in addition:
 * ComputeQSource (main/phys.c:2345-2395) and Corrector (main/phys.c:2301-2333). */
typedef struct sgo_ext {
  const int *normal;   /* [Nc*maxfaces] gridT.normal (+1 / -1)                   */
  const int *grad;     /* [2*Ne] gridT.grad, the two cells of each edge           */
  const int *edgep;    /* gridT.edgep: computational edges [edgedist[0], edgedist[1]) */
  const int *edgedist; /* [2]                                                     */
  const int *etop;     /* [Ne] gridT.etop                                          */
} sgo_ext;

/* The vertical-grid fields of UpdateDZ (main/phys.c:816-941) and SetFluxHeight
 * (main/phys.c:4338-4435). */
typedef struct sgo_vgrid {
  const double *dz;    /* [Nkmax] gridT.dz, layer thicknesses                    */
  const double *dv;    /* [Nc] gridT.dv, depth                                   */
  const double *dzbot; /* [Nc] gridT.dzbot (read when smoothbot != 0)            */
  const int *Nkc;      /* [Ne] gridT.Nkc, levels stored per dzf row (>= Nke)      */
  double smoothbot;    /* gridT.smoothbot                                          */
  double dzsmall;      /* gridT.dzsmall                                            */
} sgo_vgrid;

/* Ragged layouts of the step fields: u, utmp2 per edge with Nke[j] levels (as
 * dzf); w, wtmp2 per cell with Nk[i]+1 levels (offsets the prefix sum of
 * Nk+1); src, q, qc per cell with Nk[i] levels (as dzz). */

/* ---- the restatement (cg_oracle.c) ---- */
void sgo_cgsolveq(const sgo_grid *g, const double *D, double *q, double *src, double *c,
                  const sgo_prop *p, sgo_result *res);
void sgo_cgsolve(const sgo_grid *g, const double *D, double *h, double *htmp,
                 const sgo_prop *p, sgo_result *res);
/* single operator pieces, for kernel-level parity */
void sgo_qcoefficients(const sgo_grid *g, const double *D, const double *c, int qprecond,
                       double *coef, double *fcoef);
void sgo_operator_q(const sgo_grid *g, const double *D, const double *coef,
                    const double *x, double *y);
void sgo_operator_qc(const sgo_grid *g, const double *coef, const double *fcoef,
                     const double *x, double *y);
void sgo_condition_q(const sgo_grid *g, const double *D, double *c);
void sgo_preconditioner(const sgo_grid *g, const double *coef, const double *x, double *xc);
void sgo_hcoefficients(const sgo_grid *g, const double *D, const sgo_prop *p,
                       double *hcoef, double *hfcoef);
void sgo_operator_h(const sgo_grid *g, const double *hcoef, const double *hfcoef,
                    const double *x, double *y);
void sgo_compute_qsource(const sgo_grid *g, const sgo_ext *x, const double *u, const double *utmp2,
                         const double *w, const double *wtmp2, const sgo_prop *p, double *src, double *D);
void sgo_corrector(const sgo_grid *g, const sgo_ext *x, const double *qc, const double *D,
                   const sgo_prop *p, double *u, double *w, double *q);
/* UpdateDZ with option 0 (the per-step call, main/phys.c:3024): ctop, etop and
   dzz (rows of Nk) are updated in place from h; the old values go to ctopold,
   etopold, dzzold.  g->ctop and g->dzz are not read. */
void sgo_update_dz(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h, int linearFS,
                   int *ctop, int *etop, double *dzz, int *ctopold, int *etopold, double *dzzold);
/* SetFluxHeight: dzf (rows of Nkc levels) from u, dzz, h; dzz's bottom level is
   adjusted in place when smoothbot != 0.  x->etop and x->grad are read;
   g->dzz and g->dzf are not. */
void sgo_set_flux_height(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h,
                         const double *u, double *dzz, double *dzf);

/* ---- the reference itself (ref_harness.c, oracle/_ref only) ---- */
void ref_cgsolveq(const sgo_grid *g, const double *D, double *q, double *src, double *c,
                  const sgo_prop *p, sgo_result *res);
void ref_cgsolve(const sgo_grid *g, const double *D, double *h, double *htmp,
                 const sgo_prop *p, sgo_result *res);
void ref_qcoefficients(const sgo_grid *g, const double *D, const double *c, int qprecond,
                       double *coef, double *fcoef);
void ref_operator_q(const sgo_grid *g, const double *D, const double *coef,
                    const double *x, double *y);
void ref_operator_qc(const sgo_grid *g, const double *coef, const double *fcoef,
                     const double *x, double *y);
void ref_condition_q(const sgo_grid *g, const double *D, double *c);
void ref_preconditioner(const sgo_grid *g, const double *coef, const double *x, double *xc);
void ref_hcoefficients(const sgo_grid *g, const double *D, const sgo_prop *p,
                       double *hcoef, double *hfcoef);
void ref_operator_h(const sgo_grid *g, const double *hcoef, const double *hfcoef,
                    const double *x, double *y);
void ref_compute_qsource(const sgo_grid *g, const sgo_ext *x, const double *u, const double *utmp2,
                         const double *w, const double *wtmp2, const sgo_prop *p, double *src, double *D);
void ref_corrector(const sgo_grid *g, const sgo_ext *x, const double *qc, const double *D,
                   const sgo_prop *p, double *u, double *w, double *q);
void ref_update_dz(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h, int linearFS,
                   int *ctop, int *etop, double *dzz, int *ctopold, int *etopold, double *dzzold);
void ref_set_flux_height(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h,
                         const double *u, double *dzz, double *dzf);

#ifdef __cplusplus
}
#endif
#endif
