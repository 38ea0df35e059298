/*
 * cg_oracle.c -- TEST INFRASTRUCTURE ONLY (the "port" oracle).
 *
 * A plain-C restatement, on flat arrays, of the SUNTANS elliptic solves:
 * the nonhydrostatic pressure PCG (CGSolveQ and its helpers) and the
 * free-surface PCG (CGSolve and its helpers) from the reference's main/phys.c,
 * plus the Thomas solver from main/util.c.  Every function cites the reference
 * lines it follows.  The operation order of each floating-point expression is
 * the reference's, and the file is compiled with -ffp-contract=off, so on the
 * same inputs it returns the same bits as the reference built with gcc -O2
 * (tests/test_oracle.py checks this against oracle/_ref where the reference
 * sources are present, and against the committed golden vectors everywhere).
 *
 * Deviations from the reference, all at the call boundary, none in arithmetic:
 *  - the qprecond=1 preconditioner buffer c is the caller's own array; in the
 *    reference the call site passes phys->stmp3, which is also the residual r
 *    inside CGSolveQ (main/phys.c:1280 with main/phys.c:2419), so the final
 *    rescale divides by the converged residual.  Here c never aliases r.
 *  - scratch arrays are private to each call instead of physT fields.
 *
 * The product never links this file; the CUDA path is checked against it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "cg_oracle.h"

/* Wall-clock seconds (CLOCK_MONOTONIC), for the timing fields of sgo_result. */
static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
  long *coff;   /* [Nc+1] offsets of cell columns in the ragged arrays */
  long *eoff;   /* [Ne+1] offsets of edge columns in dzf               */
  long n3;      /* sum(Nk)                                             */
} layout_t;

static void layout_make(const sgo_grid *g, layout_t *L) {
  int i, j;
  L->coff = (long *)malloc(sizeof(long) * (g->Nc + 1));
  L->eoff = (long *)malloc(sizeof(long) * (g->Ne + 1));
  L->coff[0] = 0;
  for (i = 0; i < g->Nc; i++) L->coff[i + 1] = L->coff[i] + g->Nk[i];
  L->eoff[0] = 0;
  for (j = 0; j < g->Ne; j++) L->eoff[j + 1] = L->eoff[j] + g->Nke[j];
  L->n3 = L->coff[g->Nc];
}
static void layout_free(layout_t *L) { free(L->coff); free(L->eoff); }

#define X3(a, i, k) (a)[L->coff[(i)] + (k)]
#define DZZ(i, k) g->dzz[L->coff[(i)] + (k)]
#define DZF(j, k) g->dzf[L->eoff[(j)] + (k)]
/* fcoef row (i,nf) has Nk[i] entries and starts at maxfaces*coff[i] + nf*Nk[i] */
#define FC(i, nf, k) fcoef[(long)g->maxfaces * L->coff[(i)] + (long)(nf) * g->Nk[(i)] + (k)]

/* Summation order of the inner products.  0 (the default) is the reference's
   sequential sum in cellp order.  1 sums the same products pairwise (recursive
   halving of the sequence); it exists only so that the tests can measure how
   far a solve's iteration count moves when nothing but the order of the
   inner products' additions changes -- a parallel device reduction cannot
   reproduce the sequential order. */
static int g_sum_order = 0;
void sgo_set_sum_order(int order) { g_sum_order = order; }

static double pairwise_sum(const double *t, long n) {
  long h;
  if (n <= 0) return 0.0;
  if (n == 1) return t[0];
  h = n / 2;
  return pairwise_sum(t, h) + pairwise_sum(t + h, n - h);
}

/* Inner product over computational cells: main/phys.c:3304-3319 (InnerProduct3).
   Sequential sum in cellp order; the serial MPI_Reduce/MPI_Bcast are copies. */
static double inner3(const sgo_grid *g, const layout_t *L, const double *x, const double *y) {
  double mysum = 0;
  int iptr, i, k;
  if (g_sum_order == 1) {
    double *t = (double *)malloc(sizeof(double) * (L->n3 + 1));
    long n = 0;
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) t[n++] = X3(x, i, k) * X3(y, i, k);
    }
    mysum = pairwise_sum(t, n);
    free(t);
    return mysum;
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) mysum += X3(x, i, k) * X3(y, i, k);
  }
  return mysum;
}

/* main/phys.c:3280-3294 (InnerProduct) */
static double inner2(const sgo_grid *g, const double *x, const double *y) {
  double mysum = 0;
  int iptr, i;
  if (g_sum_order == 1) {
    double *t = (double *)malloc(sizeof(double) * (g->Nc + 1));
    long n = 0;
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      t[n++] = x[i] * y[i];
    }
    mysum = pairwise_sum(t, n);
    free(t);
    return mysum;
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    mysum += x[i] * y[i];
  }
  return mysum;
}

static int kmin_of(const sgo_grid *g, int i, int nc) {
  return g->ctop[nc] > g->ctop[i] ? g->ctop[nc] : g->ctop[i];
}

/* QCoefficients: main/phys.c:3420-3471. coef has the ragged cell layout. */
static void qcoef_impl(const sgo_grid *g, const layout_t *L, const double *D, const double *c,
                       int qprecond, double *coef, double *fcoef) {
  int iptr, i, k, nf, nc, ne, kmin;
  if (qprecond == 1) {
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      X3(coef, i, g->ctop[i]) = g->Ac[i] / DZZ(i, g->ctop[i]) / X3(c, i, g->ctop[i]);
      for (k = g->ctop[i] + 1; k < g->Nk[i]; k++)
        X3(coef, i, k) = 2 * g->Ac[i] / (DZZ(i, k) + DZZ(i, k - 1)) / (X3(c, i, k) * X3(c, i, k - 1));
      for (nf = 0; nf < g->nfaces[i]; nf++)
        if ((nc = g->neigh[i * g->maxfaces + nf]) != -1) {
          ne = g->face[i * g->maxfaces + nf];
          kmin = kmin_of(g, i, nc);
          for (k = kmin; k < g->Nke[ne]; k++)
            FC(i, nf, k) = DZZ(i, k) * D[ne] / (X3(c, i, k) * X3(c, nc, k));
        }
    }
  } else {
    /* the reference loops over all Nc cells here, not only computational ones */
    for (i = 0; i < g->Nc; i++) {
      X3(coef, i, g->ctop[i]) = g->Ac[i] / DZZ(i, g->ctop[i]);
      for (k = g->ctop[i] + 1; k < g->Nk[i]; k++)
        X3(coef, i, k) = 2 * g->Ac[i] / (DZZ(i, k) + DZZ(i, k - 1));
    }
  }
}

/* OperatorQ: main/phys.c:3486-3536 */
static void opq_impl(const sgo_grid *g, const layout_t *L, const double *D, const double *coef,
                     const double *x, double *y) {
  int iptr, i, k, nf, nc, ne, kmin;
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(y, i, k) = 0;
    for (nf = 0; nf < g->nfaces[i]; nf++)
      if ((nc = g->neigh[i * g->maxfaces + nf]) != -1) {
        ne = g->face[i * g->maxfaces + nf];
        kmin = kmin_of(g, i, nc);
        for (k = kmin; k < g->Nke[ne]; k++)
          X3(y, i, k) += (X3(x, nc, k) - X3(x, i, k)) * DZF(ne, k) * D[ne];
      }
    for (k = g->ctop[i] + 1; k < g->Nk[i] - 1; k++)
      X3(y, i, k) += X3(coef, i, k) * X3(x, i, k - 1) - (X3(coef, i, k) + X3(coef, i, k + 1)) * X3(x, i, k) +
                     X3(coef, i, k + 1) * X3(x, i, k + 1);
    if (g->ctop[i] < g->Nk[i] - 1) {
      k = g->ctop[i];
      X3(y, i, k) += (-2 * X3(coef, i, k) - X3(coef, i, k + 1)) * X3(x, i, k) + X3(coef, i, k + 1) * X3(x, i, k + 1);
      k = g->Nk[i] - 1;
      X3(y, i, k) += X3(coef, i, k) * X3(x, i, k - 1) - X3(coef, i, k) * X3(x, i, k);
    } else
      X3(y, i, g->ctop[i]) -= 2.0 * X3(coef, i, g->ctop[i]) * X3(x, i, g->ctop[i]);
  }
}

/* OperatorQC: main/phys.c:3364-3409 */
static void opqc_impl(const sgo_grid *g, const layout_t *L, const double *coef, const double *fcoef,
                      const double *x, double *y) {
  int iptr, i, k, nf, nc, ne, kmin;
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(y, i, k) = -X3(x, i, k);
    for (nf = 0; nf < g->nfaces[i]; nf++)
      if ((nc = g->neigh[i * g->maxfaces + nf]) != -1) {
        ne = g->face[i * g->maxfaces + nf];
        kmin = kmin_of(g, i, nc);
        for (k = kmin; k < g->Nke[ne]; k++) X3(y, i, k) += X3(x, nc, k) * FC(i, nf, k);
      }
    for (k = g->ctop[i] + 1; k < g->Nk[i] - 1; k++)
      X3(y, i, k) += X3(coef, i, k) * X3(x, i, k - 1) + X3(coef, i, k + 1) * X3(x, i, k + 1);
    if (g->ctop[i] < g->Nk[i] - 1) {
      k = g->ctop[i];
      X3(y, i, k) += X3(coef, i, k + 1) * X3(x, i, k + 1);
      k = g->Nk[i] - 1;
      X3(y, i, k) += X3(coef, i, k) * X3(x, i, k - 1);
    }
  }
}

/* ConditionQ: main/phys.c:3629-3687.  a[] is the reference's phys->a scratch. */
static void condq_impl(const sgo_grid *g, const layout_t *L, const double *D, double *x) {
  int iptr, i, k, nf, nc, ne, kmin;
  double *a = (double *)malloc(sizeof(double) * (g->Nkmax + 2));
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(x, i, k) = 0;
    for (nf = 0; nf < g->nfaces[i]; nf++)
      if ((nc = g->neigh[i * g->maxfaces + nf]) != -1) {
        ne = g->face[i * g->maxfaces + nf];
        kmin = kmin_of(g, i, nc);
        for (k = kmin; k < g->Nke[ne]; k++) X3(x, i, k) += DZZ(i, k) * D[ne];
      }
    a[g->ctop[i]] = g->Ac[i] / DZZ(i, g->ctop[i]);
    for (k = g->ctop[i] + 1; k < g->Nk[i]; k++) a[k] = 2 * g->Ac[i] / (DZZ(i, k) + DZZ(i, k - 1));
    for (k = g->ctop[i] + 1; k < g->Nk[i] - 1; k++) X3(x, i, k) += (a[k] + a[k + 1]);
    if (g->ctop[i] < g->Nk[i] - 1) {
      k = g->ctop[i];
      X3(x, i, k) += 2 * a[k] + a[k + 1];
      k = g->Nk[i] - 1;
      X3(x, i, k) += a[k];
    }
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) {
      if (X3(x, i, k) <= 0) X3(x, i, k) = 1;
      X3(x, i, k) = sqrt(X3(x, i, k));
    }
  }
  free(a);
}

/* TriSolve: main/util.c:185-203 (Thomas algorithm; overwrites b and d). */
static void trisolve(double *a, double *b, double *c, double *d, double *u, int N) {
  int k;
  for (k = 1; k < N; k++) {
    b[k] -= a[k] * c[k - 1] / b[k - 1];
    d[k] -= a[k] * d[k - 1] / b[k - 1];
  }
  u[N - 1] = d[N - 1] / b[N - 1];
  for (k = N - 2; k >= 0; k--) u[k] = d[k] / b[k] - c[k] * u[k + 1] / b[k];
}

/* Preconditioner: main/phys.c:3577-3619 */
static void precond_impl(const sgo_grid *g, const layout_t *L, const double *coef, const double *x,
                         double *xc) {
  int iptr, i, k, n = g->Nkmax + 2;
  double *a = (double *)calloc(n, sizeof(double)), *b = (double *)calloc(n, sizeof(double));
  double *c = (double *)calloc(n, sizeof(double)), *d = (double *)calloc(n, sizeof(double));
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    if (g->ctop[i] < g->Nk[i] - 1) {
      for (k = g->ctop[i] + 1; k < g->Nk[i] - 1; k++) {
        a[k] = X3(coef, i, k);
        b[k] = -X3(coef, i, k) - X3(coef, i, k + 1);
        c[k] = X3(coef, i, k + 1);
        d[k] = X3(x, i, k);
      }
      k = g->ctop[i];
      b[k] = -2 * X3(coef, i, k) - X3(coef, i, k + 1);
      c[k] = X3(coef, i, k + 1);
      d[k] = X3(x, i, k);
      k = g->Nk[i] - 1;
      a[k] = X3(coef, i, k);
      b[k] = -X3(coef, i, k);
      d[k] = X3(x, i, k);
      trisolve(&a[g->ctop[i]], &b[g->ctop[i]], &c[g->ctop[i]], &d[g->ctop[i]], &X3(xc, i, g->ctop[i]),
               g->Nk[i] - g->ctop[i]);
    } else
      X3(xc, i, g->ctop[i]) = -0.5 * X3(x, i, g->ctop[i]) / X3(coef, i, g->ctop[i]);
  }
  free(a); free(b); free(c); free(d);
}

/* CGSolveQ: main/phys.c:2411-2550 (x = q, p = src, z, r, rtmp as scratch). */
void sgo_cgsolveq(const sgo_grid *g, const double *D, double *q, double *src, double *c,
                  const sgo_prop *pr, sgo_result *res) {
  layout_t Lv, *L = &Lv;
  int iptr, i, k, n, niters, executed = 0;
  double mu, nu, alpha, alpha0, eps, eps0;
  double *x = q, *p = src, *z, *r, *rtmp, *coef, *fcoef;
  double t0 = now_s(), t1;
  layout_make(g, L);
  z = (double *)calloc(L->n3 + 1, sizeof(double));
  r = (double *)calloc(L->n3 + 1, sizeof(double));
  rtmp = (double *)calloc(L->n3 + 1, sizeof(double));
  coef = (double *)calloc(L->n3 + 1, sizeof(double));
  fcoef = (double *)calloc((size_t)g->maxfaces * L->n3 + 1, sizeof(double));

  if (pr->qprecond == 1) {
    condq_impl(g, L, D, c);
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) {
        X3(p, i, k) /= X3(c, i, k);
        X3(x, i, k) *= X3(c, i, k);
      }
    }
  }
  niters = pr->qmaxiters;
  qcoef_impl(g, L, D, c, pr->qprecond, coef, fcoef);

  if (pr->qprecond == 1) opqc_impl(g, L, coef, fcoef, x, z);
  else opq_impl(g, L, D, coef, x, z);
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(r, i, k) = X3(p, i, k) - X3(z, i, k);
  }
  if (pr->qprecond == 2) {
    precond_impl(g, L, coef, r, rtmp);
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(p, i, k) = X3(rtmp, i, k);
    }
    alpha = alpha0 = inner3(g, L, r, rtmp);
  } else {
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(p, i, k) = X3(r, i, k);
    }
    alpha = alpha0 = inner3(g, L, r, r);
  }
  if (!pr->resnorm) alpha0 = 1;
  if (pr->qprecond == 2) eps = eps0 = inner3(g, L, r, r);
  else eps = eps0 = alpha0;
  t1 = now_s();

  for (n = 0; n < niters && eps != 0; n++) {
    executed++;
    if (pr->qprecond == 1) opqc_impl(g, L, coef, fcoef, p, z);
    else opq_impl(g, L, D, coef, p, z);
    mu = 1 / alpha;
    nu = alpha / inner3(g, L, p, z);
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) {
        X3(x, i, k) += nu * X3(p, i, k);
        X3(r, i, k) -= nu * X3(z, i, k);
      }
    }
    if (pr->qprecond == 2) {
      precond_impl(g, L, coef, r, rtmp);
      alpha = inner3(g, L, r, rtmp);
      mu *= alpha;
      for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
        i = g->cellp[iptr];
        for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(p, i, k) = X3(rtmp, i, k) + mu * X3(p, i, k);
      }
    } else {
      alpha = inner3(g, L, r, r);
      mu *= alpha;
      for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
        i = g->cellp[iptr];
        for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(p, i, k) = X3(r, i, k) + mu * X3(p, i, k);
      }
    }
    if (pr->qprecond == 2) eps = inner3(g, L, r, r);
    else eps = alpha;
    if (sqrt(eps / eps0) < pr->qepsilon) break;
  }
  if (pr->qprecond == 1) {
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(x, i, k) /= X3(c, i, k);
    }
  }
  if (res) {
    res->niters = executed; res->eps = eps; res->eps0 = eps0;
    res->t_setup = t1 - t0; res->t_loop = now_s() - t1;
  }
  free(z); free(r); free(rtmp); free(coef); free(fcoef);
  layout_free(L);
}

/* HCoefficients: main/phys.c:3252-3269 */
static void hcoef_impl(const sgo_grid *g, const double *D, const sgo_prop *pr, double *coef, double *fcoef) {
  int iptr, i, nf, ne;
  double tmp = pr->grav * pow(pr->theta * pr->dt, 2);
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    coef[i] = g->Ac[i];
    for (nf = 0; nf < g->nfaces[i]; nf++)
      if (g->neigh[i * g->maxfaces + nf] != -1) {
        ne = g->face[i * g->maxfaces + nf];
        fcoef[i * g->maxfaces + nf] = tmp * D[ne] * g->df[ne] / g->dg[ne];
        coef[i] += fcoef[i * g->maxfaces + nf];
      }
  }
}

/* OperatorH: main/phys.c:3335-3349 */
static void oph_impl(const sgo_grid *g, const double *x, double *y, const double *coef, const double *fcoef) {
  int iptr, i, nf;
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    y[i] = coef[i] * x[i];
    for (nf = 0; nf < g->nfaces[i]; nf++)
      if (g->neigh[i * g->maxfaces + nf] != -1)
        y[i] -= fcoef[i * g->maxfaces + nf] * x[g->neigh[i * g->maxfaces + nf]];
  }
}

/* CGSolve: main/phys.c:3086-3217 (x = h, p = htmp; r, rtmp, z scratch). */
void sgo_cgsolve(const sgo_grid *g, const double *D, double *h, double *htmp, const sgo_prop *pr,
                 sgo_result *res) {
  int iptr, i, n, niters, executed = 0;
  double mu, nu, eps, eps0, alpha, alpha0;
  double *x = h, *p = htmp, *r, *rtmp, *z, *hcoef, *hfcoef;
  double t0 = now_s(), t1;
  r = (double *)calloc(g->Nc + 1, sizeof(double));
  rtmp = (double *)calloc(g->Nc + 1, sizeof(double));
  z = (double *)calloc(g->Nc + 1, sizeof(double));
  hcoef = (double *)calloc(g->Nc + 1, sizeof(double));
  hfcoef = (double *)calloc((size_t)g->maxfaces * g->Nc + 1, sizeof(double));
  niters = pr->maxiters;
  hcoef_impl(g, D, pr, hcoef, hfcoef);

  /* type-3 boundary lift, main/phys.c:3102-3134 */
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) x[g->cellp[iptr]] = 0;
  oph_impl(g, x, z, hcoef, hfcoef);
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    p[i] = p[i] - z[i];
    r[i] = p[i];
    x[i] = 0;
  }
  for (iptr = g->celldist[1]; iptr < g->celldist[2]; iptr++) p[g->cellp[iptr]] = 0;

  if (pr->hprecond == 1) {
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) { /* HPreconditioner 3227-3235 */
      i = g->cellp[iptr];
      rtmp[i] = r[i] / hcoef[i];
    }
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      p[i] = rtmp[i];
    }
    alpha = alpha0 = inner2(g, r, rtmp);
  } else {
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      p[i] = r[i];
    }
    alpha = alpha0 = inner2(g, r, r);
  }
  if (!pr->resnorm) alpha0 = 1;
  if (pr->hprecond == 1) eps = eps0 = inner2(g, r, r);
  else eps = eps0 = alpha0;
  t1 = now_s();

  for (n = 0; n < niters && eps != 0 && alpha != 0; n++) {
    executed++;
    oph_impl(g, p, z, hcoef, hfcoef);
    mu = 1 / alpha;
    nu = alpha / inner2(g, p, z);
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      x[i] += nu * p[i];
      r[i] -= nu * z[i];
    }
    if (pr->hprecond == 1) {
      for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
        i = g->cellp[iptr];
        rtmp[i] = r[i] / hcoef[i];
      }
      alpha = inner2(g, r, rtmp);
      mu *= alpha;
      for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
        i = g->cellp[iptr];
        p[i] = rtmp[i] + mu * p[i];
      }
    } else {
      alpha = inner2(g, r, r);
      mu *= alpha;
      for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
        i = g->cellp[iptr];
        p[i] = r[i] + mu * p[i];
      }
    }
    if (pr->hprecond == 1) eps = inner2(g, r, r);
    else eps = alpha;
    if (sqrt(eps / eps0) < pr->epsilon) break;
  }
  if (res) {
    res->niters = executed; res->eps = eps; res->eps0 = eps0;
    res->t_setup = t1 - t0; res->t_loop = now_s() - t1;
  }
  free(r); free(rtmp); free(z); free(hcoef); free(hfcoef);
}

/* ---- single-operator entry points (kernel-level parity) ---- */
void sgo_qcoefficients(const sgo_grid *g, const double *D, const double *c, int qprecond, double *coef,
                       double *fcoef) {
  layout_t Lv; layout_make(g, &Lv);
  qcoef_impl(g, &Lv, D, c, qprecond, coef, fcoef);
  layout_free(&Lv);
}
void sgo_operator_q(const sgo_grid *g, const double *D, const double *coef, const double *x, double *y) {
  layout_t Lv; layout_make(g, &Lv);
  opq_impl(g, &Lv, D, coef, x, y);
  layout_free(&Lv);
}
void sgo_operator_qc(const sgo_grid *g, const double *coef, const double *fcoef, const double *x, double *y) {
  layout_t Lv; layout_make(g, &Lv);
  opqc_impl(g, &Lv, coef, fcoef, x, y);
  layout_free(&Lv);
}
void sgo_condition_q(const sgo_grid *g, const double *D, double *c) {
  layout_t Lv; layout_make(g, &Lv);
  condq_impl(g, &Lv, D, c);
  layout_free(&Lv);
}
void sgo_preconditioner(const sgo_grid *g, const double *coef, const double *x, double *xc) {
  layout_t Lv; layout_make(g, &Lv);
  precond_impl(g, &Lv, coef, x, xc);
  layout_free(&Lv);
}
void sgo_hcoefficients(const sgo_grid *g, const double *D, const sgo_prop *p, double *hcoef, double *hfcoef) {
  hcoef_impl(g, D, p, hcoef, hfcoef);
}
void sgo_operator_h(const sgo_grid *g, const double *hcoef, const double *hfcoef, const double *x, double *y) {
  oph_impl(g, x, y, hcoef, hfcoef);
}

/* ------------------------------------------------------------------------
 * The steps on either side of CGSolveQ in Solve (main/phys.c:1273-1287).
 * ------------------------------------------------------------------------ */

/* ComputeQSource, main/phys.c:2345-2395: src = div(u*, w*)/dt over the wet
   levels of the computational cells (zero elsewhere), and D = df/dg. */
void sgo_compute_qsource(const sgo_grid *g, const sgo_ext *x, const double *u, const double *utmp2,
                         const double *w, const double *wtmp2, const sgo_prop *p, double *src, double *D) {
  layout_t Lv, *L = &Lv;
  int i, iptr, j, k, nf, ne;
  const double thetafactor = (1 - p->theta) / p->theta;
  long *woff;
  layout_make(g, L);
  woff = (long *)malloc(sizeof(long) * (g->Nc + 1));
  woff[0] = 0;
  for (i = 0; i < g->Nc; i++) woff[i + 1] = woff[i] + g->Nk[i] + 1;
  for (i = 0; i < g->Nc; i++)                                 /* 2357-2360 */
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(src, i, k) = 0;
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++)                   /* vertical, 2369-2373 */
      X3(src, i, k) = g->Ac[i] * (w[woff[i] + k] - w[woff[i] + k + 1]) +
                      thetafactor * g->Ac[i] * (wtmp2[woff[i] + k] - wtmp2[woff[i] + k + 1]);
    for (nf = 0; nf < g->nfaces[i]; nf++) {                   /* horizontal, 2377-2386 */
      ne = g->face[i * g->maxfaces + nf];
      for (k = g->ctop[i]; k < g->Nke[ne]; k++)
        X3(src, i, k) += (u[L->eoff[ne] + k] + thetafactor * utmp2[L->eoff[ne] + k]) * DZF(ne, k) *
                         x->normal[i * g->maxfaces + nf] * g->df[ne];
    }
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(src, i, k) /= p->dt;   /* 2389-2390 */
  }
  for (j = 0; j < g->Ne; j++) D[j] = g->df[j] / g->dg[j];   /* 2392-2394 */
  free(woff);
  layout_free(L);
}

/* Corrector, main/phys.c:2301-2333: u -= dt/dg grad(qc) on the computational
   edges with D != 0 and more than one wet level, w corrected from the
   vertical gradient of qc, and q += qc on columns with more than one level. */
void sgo_corrector(const sgo_grid *g, const sgo_ext *x, const double *qc, const double *D,
                   const sgo_prop *p, double *u, double *w, double *q) {
  layout_t Lv, *L = &Lv;
  int i, iptr, j, jptr, k;
  long *woff;
  layout_make(g, L);
  woff = (long *)malloc(sizeof(long) * (g->Nc + 1));
  woff[0] = 0;
  for (i = 0; i < g->Nc; i++) woff[i + 1] = woff[i] + g->Nk[i] + 1;
  for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {     /* 2306-2312 */
    j = x->edgep[jptr];
    if (D[j] != 0 && x->etop[j] < g->Nke[j] - 1)
      for (k = x->etop[j]; k < g->Nke[j]; k++)
        u[L->eoff[j] + k] -= p->dt / g->dg[j] * (X3(qc, x->grad[2 * j], k) - X3(qc, x->grad[2 * j + 1], k));
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {    /* 2315-2322 */
    i = g->cellp[iptr];
    for (k = g->ctop[i] + 1; k < g->Nk[i]; k++)
      w[woff[i] + k] -= 2.0 * p->dt / (DZZ(i, k - 1) + DZZ(i, k)) * (X3(qc, i, k - 1) - X3(qc, i, k));
    w[woff[i] + g->ctop[i]] += 2.0 * p->dt / DZZ(i, g->ctop[i]) * X3(qc, i, g->ctop[i]);
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {    /* 2325-2331 */
    i = g->cellp[iptr];
    if (g->ctop[i] < g->Nk[i] - 1)
      for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(q, i, k) += X3(qc, i, k);
  }
  free(woff);
  layout_free(L);
}

/* ------------------------------------------------------------------------
 * The vertical grid of the current step: UpdateDZ and SetFluxHeight.
 * ------------------------------------------------------------------------ */
#define SGO_DRYCELLHEIGHT 1e-10                       /* suntans.h:31 */
static double sgo_max(double x1, double x2) { return x2 > x1 ? x2 : x1; }   /* util.c:212-217 */
static double sgo_min(double x, double y) { return x < y ? x : y; }         /* util.c:242-246 */
static double sgo_upwind(double u, double dz1, double dz2) {                 /* util.c:219-232 */
  if (fabs(u) > 0) return u > 0 ? dz2 : dz1;
  return sgo_max(dz1, dz2);
}

/* UpdateDZ, main/phys.c:816-941, option 0. */
void sgo_update_dz(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h, int linearFS,
                   int *ctop, int *etop, double *dzz, int *ctopold, int *etopold, double *dzzold) {
  layout_t Lv, *L = &Lv;
  int i, j, k, flag, ne1, ne2;
  double z;
  if (linearFS) return;                                            /* 822-824 */
  layout_make(g, L);
  for (j = 0; j < g->Ne; j++) etopold[j] = etop[j];                /* 829-837 */
  for (i = 0; i < g->Nc; i++) {
    ctopold[i] = ctop[i];
    for (k = 0; k < ctop[i]; k++) X3(dzzold, i, k) = 0;
    for (k = ctop[i]; k < g->Nk[i]; k++) X3(dzzold, i, k) = X3(dzz, i, k);
  }
  for (i = 0; i < g->Nc; i++) {                                    /* 848-853 */
    z = 0;
    for (k = 0; k < g->Nk[i]; k++) z -= v->dz[k];
    X3(dzz, i, g->Nk[i] - 1) = v->dz[g->Nk[i] - 1] + v->dv[i] + z;
  }
  if (g->Nkmax > 1) {                                              /* 857-886 */
    for (i = 0; i < g->Nc; i++) {
      z = 0;
      flag = 0;
      for (k = 0; k < g->Nk[i]; k++) {
        z -= v->dz[k];
        if (h[i] >= z) {
          if (!flag) {
            if (k == g->Nk[i] - 1) {
              X3(dzz, i, k) = h[i] + v->dv[i];
              ctop[i] = k;
            } else if (h[i] == z) {
              X3(dzz, i, k) = 0;
              ctop[i] = k + 1;
            } else {
              X3(dzz, i, k) = h[i] - z;
              ctop[i] = k;
            }
            flag = 1;
          } else {
            if (k == g->Nk[i] - 1)
              X3(dzz, i, k) = v->dz[k] + v->dv[i] + z;
            else if (z < -v->dv[i])
              X3(dzz, i, k) = 0;
            else
              X3(dzz, i, k) = v->dz[k];
          }
        } else {
          X3(dzz, i, k) = 0;
        }
      }
    }
  } else {
    for (i = 0; i < g->Nc; i++) X3(dzz, i, 0) = v->dv[i] + h[i];  /* 887-889 */
  }
  for (j = 0; j < g->Ne; j++) {                                    /* 903-914 */
    ne1 = x->grad[2 * j];
    ne2 = x->grad[2 * j + 1];
    if (ne1 == -1) etop[j] = ctop[ne2];
    else if (ne2 == -1) etop[j] = ctop[ne1];
    else if (ctop[ne1] < ctop[ne2]) etop[j] = ctop[ne1];
    else etop[j] = ctop[ne2];
  }
  layout_free(L);
}

/* SetFluxHeight, main/phys.c:4338-4435. */
void sgo_set_flux_height(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const double *h,
                         const double *u, double *dzz, double *dzf) {
  layout_t Lv, *L = &Lv;
  int i, j, k, nc1, nc2;
  long *foff;
  layout_make(g, L);
  foff = (long *)malloc(sizeof(long) * (g->Ne + 1));
  foff[0] = 0;
  for (j = 0; j < g->Ne; j++) foff[j + 1] = foff[j] + v->Nkc[j];
  for (j = 0; j < g->Ne; j++)                                      /* 4380-4383 */
    for (k = 0; k < v->Nkc[j]; k++) dzf[foff[j] + k] = 0;
  if (v->smoothbot)                                                /* 4386-4392 */
    for (i = 0; i < g->Nc; i++)
      X3(dzz, i, g->Nk[i] - 1) = sgo_max(v->dzbot[i], v->smoothbot * v->dz[g->Nk[i] - 1]);
  for (j = 0; j < g->Ne; j++) {                                    /* 4395-4426 */
    nc1 = x->grad[2 * j];
    nc2 = x->grad[2 * j + 1];
    if (nc1 == -1) nc1 = nc2;
    if (nc2 == -1) nc2 = nc1;
    for (k = 0; k < x->etop[j]; k++) dzf[foff[j] + k] = 0;
    for (k = x->etop[j]; k < g->Nke[j]; k++)
      dzf[foff[j] + k] = sgo_upwind(u[L->eoff[j] + k], X3(dzz, nc1, k), X3(dzz, nc2, k));
    k = g->Nke[j] - 1;
    if (x->etop[j] == k)
      dzf[foff[j] + k] = sgo_max(0, sgo_upwind(u[L->eoff[j] + k], h[nc1], h[nc2]) + sgo_min(v->dv[nc1], v->dv[nc2]));
    else
      dzf[foff[j] + k] = sgo_min(X3(dzz, nc1, k), X3(dzz, nc2, k));
    for (k = x->etop[j]; k < g->Nke[j]; k++)
      if (dzf[foff[j] + k] <= SGO_DRYCELLHEIGHT) dzf[foff[j] + k] = 0;
  }
  if (v->smoothbot)                                                /* 4430-4433 */
    for (i = 0; i < g->Nc; i++)
      X3(dzz, i, g->Nk[i] - 1) = sgo_max(X3(dzz, i, g->Nk[i] - 1), v->dzsmall * v->dz[g->Nk[i] - 1]);
  free(foff);
  layout_free(L);
}

/* ------------------------------------------------------------------------
 * UPredictor, main/phys.c:2579-3077.
 * ------------------------------------------------------------------------ */
#define UE(a, j, k) (a)[L->eoff[(j)] + (k)]

/* The scratch columns of the vertical solve.  The reference keeps them in
   physT (a, b, c, d, ap, am, bp, bm, each Nkmax+1 long) across edges; they are
   kept across edges here too, starting from zero, because the single-layer
   no-slip branch reads c[Nke] (2862-2871), which the edge itself never set. */
typedef struct {
  double *a, *b, *c, *d, *e1, *a0, *b0, *c0;
} ucols_t;

static void ucols_make(ucols_t *S, int n) {
  S->a = (double *)calloc(n, sizeof(double));
  S->b = (double *)calloc(n, sizeof(double));
  S->c = (double *)calloc(n, sizeof(double));
  S->d = (double *)calloc(n, sizeof(double));
  S->e1 = (double *)calloc(n, sizeof(double));
  S->a0 = (double *)calloc(n, sizeof(double));
  S->b0 = (double *)calloc(n, sizeof(double));
  S->c0 = (double *)calloc(n, sizeof(double));
}
static void ucols_free(ucols_t *S) {
  free(S->a); free(S->b); free(S->c); free(S->d); free(S->e1); free(S->a0); free(S->b0); free(S->c0);
}

/* One computational edge of the vertical solve (2656-2945). */
static void upred_edge(const sgo_grid *g, const layout_t *L, const sgo_ext *x, const sgo_upred *up,
                       const sgo_prop *p, long *woff, ucols_t *S, int j, double *utmp, double *E, double *D) {
  const double dt = p->dt, theta = 1, alpha = 1;   /* drag fully implicit (2637-2646) */
  double *a = S->a, *b = S->b, *c = S->c, *d = S->d, *e1 = S->e1, *a0 = S->a0, *b0 = S->b0, *c0 = S->c0;
  int nc1 = x->grad[2 * j], nc2 = x->grad[2 * j + 1], et = x->etop[j], nk = g->Nke[j], k, n0, n1;
  const double *u = up->u;
  if (nc1 == -1) nc1 = nc2;
  if (nc2 == -1) nc2 = nc1;
#define Z1(k) DZZ(nc1, k)
#define Z2(k) DZZ(nc2, k)
#define UU(k) UE(u, j, k)
#define UT(k) UE(utmp, j, k)
  UT(et) += 2.0 * dt * up->tau_T[j] / (Z1(et) + Z2(et));                                 /* 2662-2663 */
  if (Z1(et) == 0 && Z2(et) == 0) return;                                                /* 2667 */
  for (k = et; k < nk; k++) a[k] = b[k] = c[k] = d[k] = 0;
  for (k = et + 1; k < nk; k++)                                                         /* 2679-2683 */
    c[k] = 0.25 * (X3(up->nu_tv, nc1, k - 1) + X3(up->nu_tv, nc2, k - 1) + X3(up->nu_tv, nc1, k) +
                   X3(up->nu_tv, nc2, k) +
                   up->laxWendroff_Vertical * (X3(up->nu_lax, nc1, k - 1) + X3(up->nu_lax, nc2, k - 1) +
                                               X3(up->nu_lax, nc1, k) + X3(up->nu_lax, nc2, k)));
  for (k = et + 1; k < nk; k++)                                                         /* 2687-2690 */
    a[k] = 2.0 * (up->nu + c[k]) / (0.25 * (Z1(k) + Z2(k)) * (Z1(k - 1) + Z2(k - 1) + Z1(k) + Z2(k)));
  for (k = et; k < nk - 1; k++)                                                         /* 2692-2696 */
    b[k] = 2.0 * (up->nu + c[k + 1]) / (0.25 * (Z1(k) + Z2(k)) * (Z1(k) + Z2(k) + Z1(k + 1) + Z2(k + 1)));
  /* k is left at et when the column has one layer, as the reference's is */
  if (up->nonlinear && up->thetaM >= 0 && nk - et > 1) {                                /* 2702-2723 */
    int kk;
    if (g->ctop[nc1] > g->ctop[nc2]) { n0 = nc2; n1 = nc1; } else { n0 = nc1; n1 = nc2; }
    for (kk = 0; kk < g->ctop[n1]; kk++) d[kk] = 0;
    for (kk = g->ctop[n1]; kk < nk; kk++) d[kk] = 0.5 * (up->w[woff[n0] + kk] + up->w[woff[n1] + kk]);
    d[nk] = 0;
    for (kk = et; kk < nk; kk++) {
      a0[kk] = (alpha * 0.5 * (d[kk] - fabs(d[kk])) + 0.5 * (1 - alpha) * d[kk]) / (0.5 * (Z1(kk) + Z2(kk)));
      b0[kk] = (alpha * 0.5 * (d[kk] + fabs(d[kk]) - d[kk + 1] + fabs(d[kk + 1])) +
                0.5 * (1 - alpha) * (d[kk] - d[kk + 1])) / (0.5 * (Z1(kk) + Z2(kk)));
      c0[kk] = -(alpha * 0.5 * (d[kk + 1] + fabs(d[kk + 1])) + 0.5 * (1 - alpha) * d[kk + 1]) /
               (0.5 * (Z1(kk) + Z2(kk)));
    }
  }
  if (nk - et > 1) {                                                                     /* 2726-2771 */
    int kk;
    for (kk = et + 1; kk < nk - 1; kk++)
      UT(kk) += dt * (1 - theta) * (a[kk] * UU(kk - 1) - (a[kk] + b[kk]) * UU(kk) + b[kk] * UU(kk + 1));
    if (up->CdT[j] == -1)
      UT(et) += dt * (1 - theta) * (a[et] * -UU(et) - (a[et] + b[et]) * UU(et) + b[et] * UU(et + 1));
    else
      UT(et) += dt * (1 - theta) *
                (-(b[et] + 2.0 * up->CdT[j] * fabs(UU(et)) / (Z1(et) + Z2(et))) * UU(et) + b[et] * UU(et + 1));
    if (up->CdB[j] == -1)
      UT(nk - 1) += dt * (1 - theta) *
                    (a[nk - 1] * UU(nk - 2) - (a[nk - 1] + b[nk - 1]) * UU(nk - 1) + b[nk - 1] * -UU(nk - 1));
    else
      UT(nk - 1) += dt * (1 - theta) *
                    (a[nk - 1] * UU(nk - 2) -
                     (a[nk - 1] + 2.0 * up->CdB[j] * fabs(UU(nk - 1)) / (Z1(nk - 1) + Z2(nk - 1))) * UU(nk - 1));
  } else {                                                                               /* 2772-2798 */
    k = et;
    if (up->CdB[j] == -1)
      UT(et) -= 2.0 * dt * (1 - theta) *
                (2.0 * (2.0 * (up->nu + c[k])) * UU(et) / ((Z1(et) + Z2(et)) * (Z1(et) + Z2(et))));
    else
      UT(et) -= 2.0 * dt * (1 - theta) * (up->CdB[j]) / (Z1(et) + Z2(et)) * fabs(UU(et)) * UU(et);
    if (up->CdT[j] == -1)
      UT(et) -= 2.0 * dt * (1 - theta) *
                (2.0 * (2.0 * (up->nu + c[k])) * UU(et) / ((Z1(et) + Z2(et)) * (Z1(et) + Z2(et))));
    else
      UT(et) -= 2.0 * dt * (1 - theta) * (up->CdT[j]) / (Z1(et) + Z2(et)) * fabs(UU(et)) * UU(et);
  }
  if (up->nonlinear && up->thetaM >= 0 && nk - et > 1) {                                /* 2801-2813 */
    int kk;
    for (kk = et + 1; kk < nk - 1; kk++)
      UT(kk) -= p->dt * (1 - up->thetaM) * (a0[kk] * UU(kk - 1) + b0[kk] * UU(kk) + c0[kk] * UU(kk + 1));
    UT(et) -= p->dt * (1 - up->thetaM) * ((a0[et] + b0[et]) * UU(et) + c0[et] * UU(et + 1));
    UT(nk - 1) -= p->dt * (1 - up->thetaM) * (a0[nk - 1] * UU(nk - 2) + (b0[nk - 1] + c0[nk - 1]) * UU(nk - 1));
  }
  for (k = et; k < nk; k++) {                                                           /* 2822-2825 */
    e1[k] = 1.0;
    d[k] = UT(k);
  }
  /* k == nk here, as in the reference */
  if (nk - et > 1) {                                                                     /* 2827-2861 */
    int kk;
    c[et] = -theta * dt * b[et];
    if (up->CdT[j] == -1)
      b[et] = 1.0 + theta * dt * (a[et] + a[et + 1] + b[et]);
    else
      b[et] = 1.0 + theta * dt * (b[et] + 2.0 * up->CdT[j] * fabs(UU(et)) / (Z1(et) + Z2(et)));
    a[et] = 0;
    c[nk - 1] = 0;
    if (up->CdB[j] == -1)
      b[nk - 1] = 1.0 + theta * dt * (a[nk - 1] + b[nk - 1] + b[nk - 2]);
    else
      b[nk - 1] = 1.0 + theta * dt * (a[nk - 1] + 2.0 * up->CdB[j] * fabs(UU(nk - 1)) / (Z1(nk - 1) + Z2(nk - 1)));
    a[nk - 1] = -theta * dt * a[nk - 1];
    for (kk = et + 1; kk < nk - 1; kk++) {
      c[kk] = -theta * dt * b[kk];
      b[kk] = 1.0 + theta * dt * (a[kk] + b[kk]);
      a[kk] = -theta * dt * a[kk];
    }
  } else {                                                                               /* 2862-2887 */
    b[et] = 1.0;
    if (up->CdB[j] == -1)
      b[et] += 4.0 * theta * dt * 2.0 * (up->nu + c[k]) / ((Z1(et) + Z2(et)) * (Z1(et) + Z2(et)));
    else
      b[et] += 2.0 * theta * dt * fabs(UT(et)) / (Z1(et) + Z2(et)) * (up->CdB[j]);
    if (up->CdT[j] == -1)
      b[et] += 4.0 * theta * dt * 2.0 * (up->nu + c[k]) / ((Z1(et) + Z2(et)) * (Z1(et) + Z2(et)));
    else
      b[et] += 2.0 * theta * dt * fabs(UT(et)) / (Z1(et) + Z2(et)) * (up->CdT[j]);
  }
  if (up->nonlinear && up->thetaM >= 0 && nk - et > 1) {                                /* 2890-2904 */
    int kk;
    for (kk = et + 1; kk < nk - 1; kk++) {
      a[kk] += p->dt * up->thetaM * a0[kk];
      b[kk] += p->dt * up->thetaM * b0[kk];
      c[kk] += p->dt * up->thetaM * c0[kk];
    }
    b[et] += p->dt * up->thetaM * (a0[et] + b0[et]);
    c[et] += p->dt * up->thetaM * c0[et];
    a[nk - 1] += p->dt * up->thetaM * a0[nk - 1];
    b[nk - 1] += p->dt * up->thetaM * (b0[nk - 1] + c0[nk - 1]);
  }
  for (k = 0; k < nk; k++) {                                                             /* 2922-2926 */
    a0[k] = a[k];
    b0[k] = b[k];
    c0[k] = c[k];
  }
  if (nk - et > 1) {                                                                     /* 2927-2935 */
    trisolve(a + et, b + et, c + et, d + et, &UT(et), nk - et);
    trisolve(a0 + et, b0 + et, c0 + et, e1 + et, &UE(E, j, et), nk - et);
  } else {
    UT(et) /= b[et];
    UE(E, j, et) = 1.0 / b[et];
  }
  D[j] = 0;                                                                              /* 2941-2943 */
  for (k = et; k < nk; k++) D[j] += UE(E, j, k) * DZF(j, k);
#undef Z1
#undef Z2
#undef UU
#undef UT
}

static long *woff_make(const sgo_grid *g) {
  long *woff = (long *)malloc(sizeof(long) * (g->Nc + 1));
  int i;
  woff[0] = 0;
  for (i = 0; i < g->Nc; i++) woff[i + 1] = woff[i] + g->Nk[i] + 1;
  return woff;
}

static int upred_vertical_impl(const sgo_grid *g, const layout_t *L, const sgo_ext *x, const sgo_upred *up,
                               const double *h, const sgo_prop *p, double *utmp, double *E, double *D) {
  ucols_t S;
  long *woff = woff_make(g);
  int j, jptr, k, nnan = 0;
  ucols_make(&S, g->Nkmax + 2);
  for (j = 0; j < g->Ne; j++) D[j] = 0;                                                  /* 2602-2603 */
  for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {                           /* 2626-2635 */
    int nc1, nc2;
    j = x->edgep[jptr];
    nc1 = x->grad[2 * j];
    nc2 = x->grad[2 * j + 1];
    for (k = x->etop[j]; k < g->Nke[j]; k++)
      UE(utmp, j, k) -= p->grav * (1 - p->theta) * p->dt * (h[nc1] - h[nc2]) / g->dg[j];
  }
  for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++)                            /* 2649-2945 */
    upred_edge(g, L, x, up, p, woff, &S, x->edgep[jptr], utmp, E, D);
  for (j = 0; j < g->Ne; j++)                                                            /* 2948-2954 */
    for (k = x->etop[j]; k < g->Nke[j]; k++)
      if (UE(utmp, j, k) != UE(utmp, j, k)) nnan++;
  free(woff);
  ucols_free(&S);
  return nnan;
}

int sgo_upredictor_vertical(const sgo_grid *g, const sgo_ext *x, const sgo_upred *up, const double *h,
                            const sgo_prop *p, double *utmp, double *E, double *D) {
  layout_t Lv;
  int n;
  layout_make(g, &Lv);
  n = upred_vertical_impl(g, &Lv, x, up, h, p, utmp, E, D);
  layout_free(&Lv);
  return n;
}

/* htmp = Ac h - dt sum_faces sum_k ((1-theta) u + theta utmp) df normal dzf (2964-2977) */
static void upred_rhs_impl(const sgo_grid *g, const layout_t *L, const sgo_ext *x, const sgo_upred *up,
                           const double *h, const sgo_prop *p, const double *utmp, double *htmp) {
  int iptr, i, nf, ne, normal, k;
  double sum;
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
    i = g->cellp[iptr];
    sum = 0;
    for (nf = 0; nf < g->nfaces[i]; nf++) {
      ne = g->face[i * g->maxfaces + nf];
      normal = x->normal[i * g->maxfaces + nf];
      for (k = x->etop[ne]; k < g->Nke[ne]; k++)
        sum += ((1 - p->theta) * UE(up->u, ne, k) + p->theta * UE(utmp, ne, k)) * g->df[ne] * normal * DZF(ne, k);
    }
    htmp[i] = g->Ac[i] * h[i] - p->dt * sum;
  }
}

void sgo_upredictor_rhs(const sgo_grid *g, const sgo_ext *x, const sgo_upred *up, const double *h,
                        const sgo_prop *p, const double *utmp, double *htmp) {
  layout_t Lv;
  layout_make(g, &Lv);
  upred_rhs_impl(g, &Lv, x, up, h, p, utmp, htmp);
  layout_free(&Lv);
}

/* The dry-cell clip (2993-3002) and u = U*** - g theta dt E dh/dg on the
   computational edges (3006-3019). */
static void upred_velocity_impl(const sgo_grid *g, const layout_t *L, const sgo_ext *x, const sgo_vgrid *v,
                                const sgo_prop *p, const double *utmp, const double *E, double *h,
                                unsigned char *active, double *u) {
  int i, j, jptr, k, nc1, nc2;
  for (i = 0; i < g->Nc; i++)
    if (h[i] <= -v->dv[i] + SGO_DRYCELLHEIGHT) {
      h[i] = -v->dv[i] + SGO_DRYCELLHEIGHT;
      active[i] = 0;
    } else {
      active[i] = 1;
    }
  for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {
    j = x->edgep[jptr];
    nc1 = x->grad[2 * j];
    nc2 = x->grad[2 * j + 1];
    for (k = x->etop[j]; k < g->Nke[j]; k++)
      UE(u, j, k) = UE(utmp, j, k) - p->grav * p->theta * p->dt * UE(E, j, k) * (h[nc1] - h[nc2]) / g->dg[j];
    if (x->etop[j] == g->Nke[j] - 1 && DZZ(nc1, x->etop[j]) == 0 && DZZ(nc2, x->etop[j]) == 0)
      UE(u, j, x->etop[j]) = 0;
  }
}

void sgo_upredictor_velocity(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_prop *p,
                             const double *utmp, const double *E, double *h, unsigned char *active, double *u) {
  layout_t Lv;
  layout_make(g, &Lv);
  upred_velocity_impl(g, &Lv, x, v, p, utmp, E, h, active, u);
  layout_free(&Lv);
}

/* u = utmp on type-2 edges (3046-3051); on each mark-3 face of a type-3 cell,
   the flux that closes the cell's continuity at every level (3055-3076).  The
   reference reads u[face][k] of the cell's other faces for k up to the
   mark-3 edge's Nke; where another face has fewer levels that read is past
   its row, and here it counts as 0. */
static void upred_boundary_impl(const sgo_grid *g, const layout_t *L, const sgo_ext *x, const sgo_ubnd *b,
                                const double *utmp, double *u) {
  int j, jptr, k, iptr, i, nf, nf1, ne, f1;
  double sum;
  for (jptr = b->edgedist[2]; jptr < b->edgedist[3]; jptr++) {
    j = b->edgep[jptr];
    for (k = x->etop[j]; k < g->Nke[j]; k++) UE(u, j, k) = UE(utmp, j, k);
  }
  for (iptr = g->celldist[1]; iptr < g->celldist[2]; iptr++) {
    i = g->cellp[iptr];
    for (nf = 0; nf < g->nfaces[i]; nf++) {
      ne = g->face[i * g->maxfaces + nf];
      if (b->mark[ne] != 3) continue;
      for (k = x->etop[ne]; k < g->Nke[ne]; k++) {
        UE(u, ne, k) = 0;
        sum = 0;
        for (nf1 = 0; nf1 < g->nfaces[i]; nf1++) {
          f1 = g->face[i * g->maxfaces + nf1];
          if (k < g->Nke[f1]) sum += UE(u, f1, k) * g->df[f1] * x->normal[i * g->maxfaces + nf1];
        }
        UE(u, ne, k) = -sum / g->df[ne] / x->normal[i * g->maxfaces + nf];
      }
    }
  }
}

void sgo_upredictor_boundary(const sgo_grid *g, const sgo_ext *x, const sgo_ubnd *b, const double *utmp,
                             double *u) {
  layout_t Lv;
  layout_make(g, &Lv);
  upred_boundary_impl(g, &Lv, x, b, utmp, u);
  layout_free(&Lv);
}

int sgo_upredictor(const sgo_grid *g, const sgo_ext *x, const sgo_vgrid *v, const sgo_upred *up,
                   const sgo_ubnd *b, const sgo_prop *p, double *u, double *h, double *utmp, double *E,
                   double *D, int *ctop, int *etop, double *dzz, unsigned char *active, sgo_result *res) {
  layout_t Lv, *L = &Lv;
  sgo_grid G = *g;
  sgo_ext X = *x;
  int i, j, jptr, k, nnan;
  int *ctopold = (int *)malloc(sizeof(int) * (g->Nc + 1));
  int *etopold = (int *)malloc(sizeof(int) * (g->Ne + 1));
  double *dzzold, *htmp = (double *)malloc(sizeof(double) * (g->Nc + 1));
  layout_make(g, L);
  dzzold = (double *)malloc(sizeof(double) * (L->n3 + 1));
  G.ctop = ctop;
  G.dzz = dzz;
  X.etop = etop;
  nnan = upred_vertical_impl(&G, L, &X, up, h, p, utmp, E, D);
  /* BoundaryVelocities without NetCDF data (boundaries.c:179-270) */
  for (i = g->celldist[1]; i < g->celldist[2]; i++) h[g->cellp[i]] = 0;
  sgo_update_dz(&G, &X, v, h, 0, ctop, etop, dzz, ctopold, etopold, dzzold);
  /* OpenBoundaryFluxes (boundaries.c:41-58) with zero boundary velocities */
  for (jptr = b->edgedist[2]; jptr < b->edgedist[5]; jptr++) {
    j = b->edgep[jptr];
    for (k = etop[j]; k < g->Nke[j]; k++) UE(utmp, j, k) = 0.0 * b->n1[j] + 0.0 * b->n2[j];
  }
  upred_rhs_impl(&G, L, &X, up, h, p, utmp, htmp);
  sgo_cgsolve(&G, D, h, htmp, p, res);
  upred_velocity_impl(&G, L, &X, v, p, utmp, E, h, active, u);
  sgo_update_dz(&G, &X, v, h, 0, ctop, etop, dzz, ctopold, etopold, dzzold);
  upred_boundary_impl(&G, L, &X, b, utmp, u);
  free(ctopold);
  free(etopold);
  free(dzzold);
  free(htmp);
  layout_free(L);
  return nnan;
}

/* ------------------------------------------------------------------------
 * WPredictor, main/phys.c:2025-2287, for grids without type-2 / type-4 edges
 * and nonlinear 0 or 1.  The reference keeps its scratch column a (phys->a)
 * across cells; with conserveMomentum it reads a[k] for levels above the
 * cell's top (2137-2138), so the column is kept across cells here too.
 * Where a cell is deeper than a face's edge the reference reads phys->ut and
 * utmp2 past the edge's Nke levels (2131-2133), memory nothing in the step
 * writes (zero at allocation); those terms are 0 here.
 * ------------------------------------------------------------------------ */
int sgo_wpredictor(const sgo_grid *g, const sgo_ext *x, const sgo_wpred *wp, const sgo_prop *p, double *w,
                   double *Cn_W, double *Cn_W2) {
  layout_t Lv, *L = &Lv;
  long *woff;
  int i, iptr, j, jptr, k, nf, ne, nc1, nc2, kmin;
  double fab1, fab2, fab3, *a, *b, *c, *wtmp, *stmp, *wc, *ut;
  const double dt = p->dt;
  if (wp->nonlinear != 0 && wp->nonlinear != 1) return -1;
  layout_make(g, L);
  woff = woff_make(g);
#define W(i, k) w[woff[(i)] + (k)]
  a = (double *)calloc(g->Nkmax + 2, sizeof(double));
  b = (double *)calloc(g->Nkmax + 2, sizeof(double));
  c = (double *)calloc(g->Nkmax + 2, sizeof(double));
  wtmp = (double *)calloc(L->n3 + 1, sizeof(double));
  stmp = (double *)calloc(L->n3 + 1, sizeof(double));
  wc = (double *)calloc(L->n3 + 1, sizeof(double));
  ut = (double *)calloc(L->eoff[g->Ne] + 1, sizeof(double));
  if (wp->n == 1) {                                                                /* 2044-2067 */
    fab1 = 1;
    fab2 = fab3 = 0;
    for (i = 0; i < g->Nc; i++)
      for (k = 0; k < g->Nk[i]; k++) X3(Cn_W, i, k) = X3(Cn_W2, i, k) = 0;
  } else if (wp->n == 2 || wp->AB == 2) {
    fab1 = 3.0 / 2.0;
    fab2 = -1.0 / 2.0;
    fab3 = 0;
  } else {
    fab1 = 23.0 / 12.0;
    fab2 = -4.0 / 3.0;
    fab3 = 5.0 / 12.0;
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {                     /* 2071-2089 */
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) {
      X3(wtmp, i, k) = W(i, k) + fab2 * X3(Cn_W, i, k) + fab3 * X3(Cn_W2, i, k);
      X3(Cn_W2, i, k) = X3(Cn_W, i, k);
      X3(Cn_W, i, k) = 0;
    }
    for (k = g->ctop[i] + 1; k < g->Nk[i]; k++)
      X3(wtmp, i, k) -= 2.0 * dt / (DZZ(i, k - 1) + DZZ(i, k)) * (X3(wp->q, i, k - 1) - X3(wp->q, i, k));
    X3(wtmp, i, g->ctop[i]) += 2.0 * dt / DZZ(i, g->ctop[i]) * X3(wp->q, i, g->ctop[i]);
  }
  if (wp->nonlinear) {                                                             /* 2095-2146 */
    for (i = 0; i < g->Nc; i++)
      for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(wc, i, k) = 0.5 * (W(i, k) + W(i, k + 1));
    /* GetMomentumFaceValues, first-order upwind (4879-4968) */
    for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {
      j = x->edgep[jptr];
      nc1 = x->grad[2 * j];
      nc2 = x->grad[2 * j + 1];
      kmin = g->ctop[nc1] > g->ctop[nc2] ? g->ctop[nc1] : g->ctop[nc2];
      for (k = 0; k < kmin && k < g->Nke[j]; k++) UE(ut, j, k) = 0;
      for (k = kmin; k < g->Nke[j]; k++) UE(ut, j, k) = UE(wp->utmp2, j, k) > 0 ? X3(wc, nc2, k) : X3(wc, nc1, k);
    }
    /* faces of type-3 cells: the same first-order upwind values */
    if (wp->conserveMomentum)
      for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {
        j = x->edgep[jptr];
        for (k = x->etop[j]; k < g->Nke[j]; k++) UE(ut, j, k) *= DZF(j, k);
      }
    for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {
      i = g->cellp[iptr];
      for (k = g->ctop[i]; k < g->Nk[i]; k++) a[k] = wp->conserveMomentum ? DZZ(i, k) : 1.0;
      for (nf = 0; nf < g->nfaces[i]; nf++) {
        const double nrm = x->normal[i * g->maxfaces + nf];
        ne = g->face[i * g->maxfaces + nf];
        for (k = g->ctop[i]; k < g->Nk[i] && k < g->Nke[ne]; k++)
          X3(stmp, i, k) += UE(ut, ne, k) * UE(wp->utmp2, ne, k) * g->df[ne] * nrm / (a[k] * g->Ac[i]);
        if (wp->conserveMomentum)
          for (k = x->etop[ne]; k < g->ctop[i]; k++)
            X3(stmp, i, g->ctop[i]) += UE(ut, ne, k) * UE(wp->utmp2, ne, k) * g->df[ne] * nrm / (a[k] * g->Ac[i]);
      }
      for (k = g->ctop[i]; k < g->Nk[i]; k++)    /* pow(w,2) is w*w */
        X3(stmp, i, k) += (W(i, k) * W(i, k) - W(i, k + 1) * W(i, k + 1)) / DZZ(i, k);
    }
  }
  for (jptr = x->edgedist[0]; jptr < x->edgedist[1]; jptr++) {                     /* 2159-2185 */
    j = x->edgep[jptr];
    nc1 = x->grad[2 * j];
    nc2 = x->grad[2 * j + 1];
    kmin = g->ctop[nc1] > g->ctop[nc2] ? g->ctop[nc1] : g->ctop[nc2];
    for (k = kmin; k < g->Nke[j]; k++) {
      a[k] = .5 * (wp->nu_H + 0.5 * (X3(wp->nu_lax, nc1, k) + X3(wp->nu_lax, nc2, k))) *
             (W(nc2, k) - W(nc1, k) + W(nc2, k + 1) - W(nc1, k + 1)) * g->df[j] / g->dg[j];
      X3(stmp, nc1, k) -= a[k] / g->Ac[nc1];
      X3(stmp, nc2, k) += a[k] / g->Ac[nc2];
    }
    for (k = g->Nke[j]; k < g->Nk[nc1]; k++)
      X3(stmp, nc1, k) += 0.25 * wp->CdW * fabs(W(nc1, k) + W(nc1, k + 1)) * (W(nc1, k) + W(nc1, k + 1)) * g->df[j] /
                          g->Ac[nc1];
    for (k = g->Nke[j]; k < g->Nk[nc2]; k++)
      X3(stmp, nc2, k) += 0.25 * wp->CdW * fabs(W(nc2, k) + W(nc2, k + 1)) * (W(nc2, k) + W(nc2, k + 1)) * g->df[j] /
                          g->Ac[nc2];
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {                     /* 2210-2220 */
    i = g->cellp[iptr];
    for (k = g->ctop[i] + 1; k < g->Nk[i]; k++)
      X3(Cn_W, i, k) -= dt * (DZZ(i, k - 1) * X3(stmp, i, k - 1) + DZZ(i, k) * X3(stmp, i, k)) /
                        (DZZ(i, k - 1) + DZZ(i, k));
    k = g->ctop[i];
    X3(Cn_W, i, k) -= dt * X3(stmp, i, k);
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {                     /* 2236-2241 */
    i = g->cellp[iptr];
    for (k = g->ctop[i]; k < g->Nk[i]; k++) X3(wtmp, i, k) += fab1 * X3(Cn_W, i, k);
  }
  for (iptr = g->celldist[0]; iptr < g->celldist[1]; iptr++) {                     /* 2246-2284 */
    const int ct = g->ctop[i = g->cellp[iptr]], nk = g->Nk[i];
    const double lv = wp->laxWendroff_Vertical;
    if (nk - ct > 1) {
      for (k = ct + 1; k < nk; k++) {
        a[k] = 2 * (wp->nu + lv * X3(wp->nu_lax, i, k - 1) + X3(wp->nu_tv, i, k - 1)) / DZZ(i, k - 1) /
               (DZZ(i, k) + DZZ(i, k - 1));
        b[k] = 2 * (wp->nu + lv * X3(wp->nu_lax, i, k) + X3(wp->nu_tv, i, k)) / DZZ(i, k) / (DZZ(i, k) + DZZ(i, k - 1));
      }
      b[ct] = (wp->nu + lv * X3(wp->nu_lax, i, ct) + X3(wp->nu_tv, i, ct)) / (DZZ(i, ct) * DZZ(i, ct));
      a[ct] = b[ct];
      for (k = ct + 1; k < nk; k++)
        X3(wtmp, i, k) += dt * (1 - p->theta) * (a[k] * W(i, k - 1) - (a[k] + b[k]) * W(i, k) + b[k] * W(i, k + 1));
      X3(wtmp, i, ct) += dt * (1 - p->theta) * (-(a[ct] + b[ct]) * W(i, ct) + (a[ct] + b[ct]) * W(i, ct + 1));
      for (k = ct; k < nk; k++) {
        c[k] = 1 + dt * p->theta * (a[k] + b[k]);
        a[k] *= (-dt * p->theta);
        b[k] *= (-dt * p->theta);
      }
      b[ct] += a[ct];
      trisolve(a + ct, c + ct, b + ct, &X3(wtmp, i, ct), &W(i, ct), nk - ct);
    } else {
      for (k = ct; k < nk; k++) W(i, k) = X3(wtmp, i, k);
    }
  }
#undef W
  free(a); free(b); free(c); free(wtmp); free(stmp); free(wc); free(ut); free(woff);
  layout_free(L);
  return 0;
}
