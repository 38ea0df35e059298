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
  double t_setup;      /* seconds before the iteration loop (coefficients,
                          conditioning, first residual); port only               */
  double t_loop;       /* seconds in the iteration loop; port only               */
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

/* UPredictor (main/phys.c:2579-3077): the fields it reads beyond the grid. */
typedef struct sgo_upred {
  const double *u;      /* [ne3] u at step n, rows of Nke                        */
  const double *w;      /* [nw3] w at step n, rows of Nk+1 (vertical advection)  */
  const double *tau_T;  /* [Ne] surface stress                                    */
  const double *CdT;    /* [Ne] top drag coefficient, -1 = no slip                */
  const double *CdB;    /* [Ne] bottom drag coefficient, -1 = no slip             */
  const double *nu_tv;  /* [n3] vertical eddy viscosity at cell centres           */
  const double *nu_lax; /* [n3] Lax-Wendroff viscosity                            */
  double nu;            /* propT.nu                                               */
  double laxWendroff_Vertical;
  double thetaM;        /* < 0: no implicit vertical momentum advection           */
  int nonlinear;
} sgo_upred;

/* The open-boundary part of UpdateDZ's caller: all edges ordered by mark
   (edgep, edgedist[6], main/grid.c:1666-1679), their marks and normals. */
typedef struct sgo_ubnd {
  const int *edgep;
  const int *edgedist;  /* [6] */
  const int *mark;      /* [Ne] */
  const double *n1;     /* [Ne] */
  const double *n2;     /* [Ne] */
} sgo_ubnd;

/* WPredictor (main/phys.c:2025-2287): the fields it reads beyond the grid. */
typedef struct sgo_wpred {
  const double *q;      /* [n3] nonhydrostatic pressure                           */
  const double *nu_tv;  /* [n3]                                                    */
  const double *nu_lax; /* [n3]                                                    */
  const double *utmp2;  /* [ne3] rows of Nke: the advecting face velocity          */
  double nu, nu_H, CdW, laxWendroff_Vertical;
  int nonlinear;        /* 0 or 1 (first-order upwind face values)                */
  int conserveMomentum;
  int n, AB;            /* propT.n (time step) and propT.AB (2 or 3)               */
} sgo_wpred;

/* ---- the restatement (cg_oracle.c) ---- */
void sgo_cgsolveq(const sgo_grid *g, const double *D, double *q, double *src, double *c,
                  const sgo_prop *p, sgo_result *res);
void sgo_cgsolve(const sgo_grid *g, const double *D, double *h, double *htmp,
                 const sgo_prop *p, sgo_result *res);
/* order of the inner products' additions: 0 sequential (the reference's),
   1 pairwise (tests only: measures a solve's sensitivity to that order) */
void sgo_set_sum_order(int order);
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

/* UPredictor in pieces.  _vertical: U*** in utmp (in: the horizontal source),
   E = A^{-1} 1 and D = dzf^T E on the computational edges (main/phys.c:2604-2945;
   D is zeroed on every edge, E rows of skipped edges are left alone); returns
   the number of NaN values in utmp (the reference stops on any, 2948-2954).
   _rhs: the free-surface right-hand side htmp on computational cells
   (2964-2977).  _velocity: the dry-cell clip of h and u on the computational
   edges after the solve (2991-3019).  _boundary: u on type-2 edges and on the
   mark-3 faces of type-3 cells (3046-3076). */
int sgo_upredictor_vertical(const sgo_grid *g, const sgo_ext *x, const sgo_upred *up, const double *h,
                            const sgo_prop *p, double *utmp, double *E, double *D);
void sgo_upredictor_rhs(const sgo_grid *g, const sgo_ext *x, const sgo_upred *up, const double *h,
                        const sgo_prop *p, const double *utmp, double *htmp);
void sgo_upredictor_velocity(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_prop *p,
                             const double *utmp, const double *E, double *h, unsigned char *active, double *u);
void sgo_upredictor_boundary(const sgo_grid *g, const sgo_ext *x, const sgo_ubnd *b, const double *utmp,
                             double *u);
/* The whole of UPredictor with CGSolve (cgsolver 1), for a model without
   NetCDF boundary data: BoundaryVelocities sets h = 0 at type-3 cells and
   calls UpdateDZ, OpenBoundaryFluxes sets utmp = 0*n1 + 0*n2 on edges of marks
   2-4.  ctop, etop, dzz (rows of Nk) are the state before the call and are
   updated in place; u, h, utmp, E, D as above; res = CGSolve's. */
int sgo_upredictor(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_upred *up,
                   const sgo_ubnd *b, const sgo_prop *p, double *u, double *h, double *utmp, double *E,
                   double *D, int *ctop, int *etop, double *dzz, unsigned char *active, sgo_result *res);

/* WPredictor for a grid without type-2 or type-4 edges: w (rows of Nk+1) is
   advanced on the computational cells; Cn_W and Cn_W2 (rows of Nk) are the
   Adams-Bashforth histories, updated in place.  x->edgep / edgedist are the
   computational edges, x->etop is read with conserveMomentum.  Returns 0, or
   -1 for a nonlinear scheme other than 0 and 1. */
int sgo_wpredictor(const sgo_grid *g, const sgo_ext *x, const sgo_wpred *wp, const sgo_prop *p, double *w,
                   double *Cn_W, double *Cn_W2);

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

int ref_wpredictor(const sgo_grid *g, const sgo_ext *x, const sgo_wpred *wp, const sgo_prop *p, double *w,
                   double *Cn_W, double *Cn_W2);
int ref_upredictor(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_upred *up,
                   const sgo_ubnd *b, const sgo_prop *p, double *u, double *h, double *utmp, double *E,
                   double *D, int *ctop, int *etop, double *dzz, unsigned char *active, sgo_result *res);

#ifdef __cplusplus
}
#endif
#endif
