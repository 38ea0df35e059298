/*
 * suntans_gb300.h -- C ABI of the GB300 elliptic solvers for SUNTANS.
 *
 * Drop-in replacements for the two conjugate-gradient solves of the SUNTANS
 * reference (ofringer/suntans, main/phys.c):
 *
 *   static void CGSolveQ(REAL **q, REAL **src, REAL **c, gridT *grid, physT *phys,
 *                        propT *prop, int myproc, int numprocs, MPI_Comm comm);
 *        declared main/phys.c:50-52, defined main/phys.c:2411-2550
 *   static void CGSolve(gridT *grid, physT *phys, propT *prop, int myproc,
 *                       int numprocs, MPI_Comm comm);
 *        declared main/phys.c:45-46, defined main/phys.c:3086-3217
 *
 * Every entry point takes plain pointers and sizes.  The 3-D fields are the
 * reference's own jagged arrays: row i of q, src, c and dzz points at Nk[i]
 * doubles (cell index order), row j of dzf at Nke[j] doubles.  The solves run
 * on one GPU as a single partition: the reference's halo exchanges
 * (ISendRecvCellData2D/3D, main/sendrecv.c:134-217) have nothing to exchange
 * and its MPI_Reduce + MPI_Bcast inner products (main/phys.c:3290-3291,
 * 3315-3316) become in-kernel reductions.  There is no CPU fallback: without a
 * usable CUDA device every entry point returns SGPU_NO_DEVICE.
 *
 * The adapter with the reference's own signatures (gridT/physT/propT) and the
 * two-line call-site patch of main/phys.c are in suntans_gb300/shim/.
 */
#ifndef SUNTANS_GB300_H
#define SUNTANS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (every entry point returns one) */
#define SGPU_OK 0          /* converged (or eps == 0 at start, as the reference) */
#define SGPU_MAXITER 1     /* maxiters reached without convergence; x is the last iterate */
#define SGPU_BREAKDOWN 2   /* p.Ap == 0 or a non-finite scalar; the solve stopped */
#define SGPU_TIMEOUT 3     /* a device-side barrier wait hit its time limit */
#define SGPU_OOM 4         /* device or pinned allocation failed */
#define SGPU_BAD_GRID 5    /* grid description fails validation (message: sgpu_last_error) */
#define SGPU_BAD_ARG 6     /* null pointer or out-of-range parameter */
#define SGPU_CUDA_ERROR 7  /* a CUDA call failed (message: sgpu_last_error) */
#define SGPU_NO_DEVICE 8   /* no CUDA device, or the library was built without one */
#define SGPU_TOO_LARGE 9   /* grid exceeds the fixed scratch of sgpu_cgsolve_noalloc */

/* The part of gridT (main/grid.h:32-149) the two solves read and that does not
 * change between time steps.  Arrays are copied at sgpu_create; the caller
 * keeps ownership. */
typedef struct sgpu_grid_desc {
  int Nc, Ne, maxfaces, Nkmax;
  const int *nfaces;   /* [Nc]             gridT.nfaces                         */
  const int *neigh;    /* [Nc*maxfaces]    gridT.neigh, -1 = no neighbour       */
  const int *face;     /* [Nc*maxfaces]    gridT.face                           */
  const int *Nk;       /* [Nc]             gridT.Nk                             */
  const int *Nke;      /* [Ne]             gridT.Nke                            */
  const int *cellp;    /* [celldist[2]]    gridT.cellp                          */
  const int *celldist; /* [3]              gridT.celldist                       */
  const double *Ac;    /* [Nc]             gridT.Ac                             */
  const double *df;    /* [Ne]             gridT.df                             */
  const double *dg;    /* [Ne]             gridT.dg                             */
} sgpu_grid_desc;

/* The propT fields (main/phys.h:183-203) the two solves read. */
typedef struct sgpu_props {
  int qprecond;     /* 0 none, 1 diagonal scaling (OperatorQC), 2 column tridiagonal */
  int qmaxiters;
  double qepsilon;
  int hprecond;     /* 0 none, 1 Jacobi */
  int maxiters;
  double epsilon;
  double resnorm;   /* 0: qprecond 0/1 and hprecond 0 stop on the absolute norm */
  double grav, theta, dt;
} sgpu_props;

/* Per-solve report (not in the reference, which returns void). */
typedef struct sgpu_stats {
  int status;
  int niters;        /* solver iterations executed */
  double eps, eps0;  /* last eps and its normaliser: converged iff sqrt(eps/eps0) < tol */
  double ms_solve;   /* device time of the solve kernel (CUDA events) */
  double ms_total;   /* wall time of the call, copies included */
  long long unknowns;/* N_q = sum (Nk - ctop) over computational cells, or N_h */
} sgpu_stats;

typedef struct sgpu_context sgpu_context;

/* Builds the device copy of one grid on CUDA device `device` (the context's
 * device stays current only inside calls).  Replaces nothing in the reference:
 * it is the one-time upload the reference never needed (its grid lives in host
 * memory).  Returns SGPU_BAD_GRID with a message for inconsistent input. */
int sgpu_create(const sgpu_grid_desc *grid, int device, sgpu_context **out);
int sgpu_destroy(sgpu_context *ctx);
const char *sgpu_last_error(const sgpu_context *ctx);
const char *sgpu_status_string(int status);

/* CGSolveQ drop-in (main/phys.c:2411-2550).
 *   ctop[Nc]            gridT.ctop            (changes every step)
 *   dzz[Nc][Nk]         gridT.dzz             (changes every step)
 *   dzf[Ne][Nke]        gridT.dzf             (changes every step)
 *   D[Ne]               phys->D = df/dg       (set by ComputeQSource, phys.c:2392)
 *   q[Nc][Nk]           phys->qc: warm start in, solution out (computational cells,
 *                       k in [ctop, Nk)); other entries untouched, as in the reference
 *   src[Nc][Nk]         phys->stmp: right-hand side.  The reference destroys it (uses it
 *                       as p); this call leaves it unchanged, which no caller can observe
 *   c[Nc][Nk]           preconditioner buffer: read only at type-3 boundary cells for
 *                       qprecond 1 (the reference reads whatever the buffer holds there).
 *                       Not written (the reference's buffer aliases its residual).
 */
int sgpu_cgsolveq(sgpu_context *ctx, const int *ctop, const double *const *dzz, const double *const *dzf,
                  const double *D, double *const *q, const double *const *src, const double *const *c,
                  const sgpu_props *prop, sgpu_stats *stats);

/* CGSolve drop-in (main/phys.c:3086-3217).
 *   D[Ne]      phys->D = sum_k E dzf (UPredictor, main/phys.c:2935-2937)
 *   h[Nc]      phys->h: type-3 boundary values in; solution out at computational cells
 *   htmp[Nc]   phys->htmp: right-hand side (left unchanged; the reference destroys it) */
int sgpu_cgsolve(sgpu_context *ctx, const double *D, double *h, const double *htmp,
                 const sgpu_props *prop, sgpu_stats *stats);

/* ---- the steps on either side of CGSolveQ in Solve (main/phys.c:1273-1287) ----
 * Field layouts as the reference's jagged rows: u, utmp2 and dzf per edge
 * (Nke[j] levels), w and wtmp2 per cell with Nk[i]+1 levels, q, qc, src, dzz
 * per cell (Nk[i] levels). */

/* The gridT fields these steps read beyond sgpu_grid_desc, uploaded once:
 *   normal[Nc*maxfaces] gridT.normal (+1/-1), grad[2*Ne] gridT.grad (the two
 *   cells of each edge, -1 = none), edgep[] / edgedist[2] gridT.edgep and
 *   edgedist (computational edges edgep[edgedist[0]..edgedist[1])). */
int sgpu_step_grid(sgpu_context *ctx, const int *normal, const int *grad, const int *edgep, const int *edgedist);

/* ComputeQSource drop-in (main/phys.c:2345-2395): src = div(u*, w*)/dt on the
 * wet levels of the computational cells, 0 on levels [ctop, Nk) elsewhere;
 * D = df/dg.  theta, dt are propT.theta, propT.dt.  Same bits as the reference. */
int sgpu_compute_qsource(sgpu_context *ctx, const int *ctop, const double *const *dzf, const double *const *u,
                         const double *const *utmp2, const double *const *w, const double *const *wtmp2,
                         double theta, double dt, double *const *src, double *D);

/* Corrector drop-in (main/phys.c:2301-2333): u, w and q updated in place with
 * the pressure correction qc (etop = gridT.etop, D from ComputeQSource).
 * Same bits as the reference. */
int sgpu_corrector(sgpu_context *ctx, const int *ctop, const int *etop, const double *const *dzz,
                   const double *const *qc, const double *D, double dt, double *const *u, double *const *w,
                   double *const *q);

/* The three in one call (ComputeQSource -> CGSolveQ -> Corrector, as Solve
 * runs them): the right-hand side and D are formed on the device and never
 * leave it, the solution qc stays on the device for the correction.  qc is the
 * warm start in and the solution out; u, w, q are updated in place; c as for
 * sgpu_cgsolveq.  Returns the solve's status (stats as sgpu_cgsolveq). */
int sgpu_pressure_step(sgpu_context *ctx, const int *ctop, const int *etop, const double *const *dzz,
                       const double *const *dzf, const double *const *utmp2, const double *const *wtmp2,
                       double *const *u, double *const *w, double *const *q, double *const *qc,
                       const double *const *c, const sgpu_props *prop, sgpu_stats *stats);

/* ---- the vertical grid of the step (it drives both solvers' coefficients) ---- */
typedef struct sgpu_vgrid {
  const double *dz;    /* [Nkmax] gridT.dz, layer thicknesses                        */
  const double *dv;    /* [Nc] gridT.dv, depth                                       */
  const double *dzbot; /* [Nc] gridT.dzbot (needed when smoothbot != 0)              */
  const int *Nkc;      /* [Ne] gridT.Nkc, levels stored per dzf row (>= Nke)          */
  double smoothbot;    /* gridT.smoothbot                                              */
  double dzsmall;      /* gridT.dzsmall                                                */
} sgpu_vgrid;

/* UpdateDZ drop-in for the per-step call (option 0, main/phys.c:816-941, called
 * at 3024): from the free surface h, dzz (rows of Nk), ctop and etop are updated
 * in place and their previous values written to dzzold, ctopold, etopold.
 * linearFS != 0 returns at once, as the reference.  Needs sgpu_step_grid (grad).
 * Same bits as the reference. */
int sgpu_update_dz(sgpu_context *ctx, const sgpu_vgrid *v, const double *h, int linearFS, int *ctop, int *etop,
                   double *const *dzz, int *ctopold, int *etopold, double *const *dzzold);

/* SetFluxHeight drop-in (main/phys.c:4338-4435): dzf (rows of Nkc levels) from
 * u (rows of Nke), dzz and h; with smoothbot != 0 the bottom level of dzz is
 * adjusted in place as in the reference.  Same bits as the reference. */
int sgpu_set_flux_height(sgpu_context *ctx, const sgpu_vgrid *v, const int *etop, const double *h,
                         const double *const *u, double *const *dzz, double *const *dzf);

/* ---- WPredictor (main/phys.c:2025-2287): the vertical-velocity predictor ---- */

typedef struct sgpu_wpred_fields {
  const double *const *q;      /* [Nc] rows of Nk: nonhydrostatic pressure phys->q           */
  const double *const *nu_tv;  /* [Nc] rows of Nk                                              */
  const double *const *nu_lax; /* [Nc] rows of Nk                                              */
  const double *const *utmp2;  /* [Ne] rows of Nke: advecting velocity (read when nonlinear)   */
  double nu, nu_H, CdW, laxWendroff_Vertical; /* propT                                        */
  int nonlinear;               /* 0 or 1 on the device                                         */
  int conserveMomentum;        /* 0 on the device                                              */
  int n, AB;                   /* propT.n (1 = first step) and propT.AB                        */
} sgpu_wpred_fields;

/* WPredictor drop-in for grids without type-2 or type-4 edges: w (rows of
 * Nk+1) advances on the computational cells and the Adams-Bashforth histories
 * Cn_W, Cn_W2 (rows of at least Nk) are updated in place; prop gives dt and
 * theta.  Needs sgpu_step_grid, whose edge list sets the order of the
 * horizontal-diffusion sums.  Same bits as the reference. */
int sgpu_wpredictor(sgpu_context *ctx, const int *ctop, const double *const *dzz, const sgpu_wpred_fields *f,
                    const sgpu_props *prop, double *const *w, double *const *Cn_W, double *const *Cn_W2);

/* The nonhydrostatic part of Solve in one call (main/phys.c:1271-1289):
 * WPredictor -> ComputeQSource -> CGSolveQ -> Corrector, with w, q, the
 * right-hand side, D and the correction kept in HBM between the steps.  wf
 * supplies WPredictor's viscosities and settings (its q and utmp2 are the q
 * and utmp2 given here); Cn_W / Cn_W2 are its histories, updated in place.
 * Every step but the solve has the reference's bits. */
int sgpu_nonhydrostatic_step(sgpu_context *ctx, const int *ctop, const int *etop, const double *const *dzz,
                             const double *const *dzf, const double *const *utmp2, const double *const *wtmp2,
                             const sgpu_wpred_fields *wf, double *const *u, double *const *w, double *const *q,
                             double *const *qc, const double *const *c, double *const *Cn_W, double *const *Cn_W2,
                             const sgpu_props *prop, sgpu_stats *stats);

/* ---- UPredictor (main/phys.c:2579-3077): the predictor around CGSolve ---- */

/* The edge description UPredictor's boundary steps read, once per grid: every
 * edge ordered by mark as gridT.edgep / edgedist[6] (main/grid.c:1666-1679),
 * gridT.mark, the edge normals gridT.n1 / n2, and every cell's faces and
 * their signs (gridT.face, normal).  Needs sgpu_step_grid. */
int sgpu_upredictor_grid(sgpu_context *ctx, const int *edgep, const int *edgedist, const int *mark, const double *n1,
                         const double *n2, const int *face, const int *normal);

typedef struct sgpu_upred_fields {
  const double *const *u;      /* [Ne] rows of Nke: u at step n (phys->u)                       */
  const double *const *w;      /* [Nc] rows of Nk+1: w (read when nonlinear && thetaM >= 0)     */
  const double *const *nu_tv;  /* [Nc] rows of Nk: vertical eddy viscosity                       */
  const double *const *nu_lax; /* [Nc] rows of Nk: Lax-Wendroff viscosity                        */
  const double *tau_T;         /* [Ne] surface stress                                             */
  const double *CdT;           /* [Ne] top drag coefficient, -1 = no slip                         */
  const double *CdB;           /* [Ne] bottom drag coefficient, -1 = no slip                      */
  double nu;                   /* propT.nu                                                        */
  double laxWendroff_Vertical; /* propT.laxWendroff_Vertical                                      */
  double thetaM;               /* propT.thetaM (< 0: no implicit vertical advection)              */
  int nonlinear;               /* propT.nonlinear                                                 */
} sgpu_upred_fields;

/* The vertically implicit predictor (2602-2945) on the computational edges:
 * utmp (in: the explicit horizontal source phys->utmp) becomes U***, E
 * (phys->ut) = A^{-1} [1..1] on their rows, and D = dzf^T E (0 on every other
 * edge).  h is the free surface at step n; prop gives dt, theta, grav.  Same
 * bits as the reference, except that a no-slip single-layer edge reads c = 0
 * where the reference reads a scratch value an earlier edge left (2864-2871).
 * A NaN in U*** returns SGPU_BREAKDOWN (the reference stops the run). */
int sgpu_upredictor_vertical(sgpu_context *ctx, const int *ctop, const int *etop, const double *const *dzz,
                             const double *const *dzf, const double *h, const sgpu_upred_fields *f,
                             const sgpu_props *prop, double *const *utmp, double *const *E, double *D);

/* The free-surface right-hand side CGSolve reads (2964-2977), on the
 * computational cells: htmp = Ac h - dt sum_faces sum_k ((1-theta) u + theta
 * utmp) df normal dzf.  Same bits as the reference. */
int sgpu_upredictor_rhs(sgpu_context *ctx, const int *etop, const double *const *dzf, const double *const *u,
                        const double *const *utmp, const double *h, const sgpu_props *prop, double *htmp);

/* After CGSolve (2991-3076): the dry-cell clip of h (active[i] = 0 where it
 * clips, 1 elsewhere; the caller zeroes phys->s at the bottom of those
 * cells), u = U*** - g theta dt E (h1 - h2)/dg on the computational edges,
 * UpdateDZ (ctop, etop, dzz in place), u = utmp on type-2 edges and the
 * continuity flux on the mark-3 faces of type-3 cells.  Needs
 * sgpu_upredictor_grid.  Same bits as the reference. */
int sgpu_upredictor_finish(sgpu_context *ctx, const sgpu_vgrid *v, const sgpu_props *prop, int *ctop, int *etop,
                           double *const *dzz, const double *const *utmp, const double *const *E, double *h,
                           unsigned char *active, double *const *u);

/* The whole UPredictor on the device, with CGSolve (cgsolver 1) in between,
 * for a model without NetCDF boundary data: the boundary step sets h = 0 on
 * type-3 cells, runs UpdateDZ and sets utmp = 0 n1 + 0 n2 on edges of marks
 * 2-4 (BoundaryVelocities / OpenBoundaryFluxes, boundaries.c:41-58, 179-270).
 * Between the upload of the step's fields and the download of u, h, utmp, E,
 * D, ctop, etop, dzz and active everything stays in HBM.  Returns CGSolve's
 * status. */
int sgpu_upredictor(sgpu_context *ctx, const sgpu_vgrid *v, const sgpu_upred_fields *f, const sgpu_props *prop,
                    int *ctop, int *etop, double *const *dzz, const double *const *dzf, double *const *u, double *h,
                    double *const *utmp, double *const *E, double *D, unsigned char *active, sgpu_stats *stats);

/* Staged forms of the same two solves, for callers that keep inputs resident:
 * upload (host -> HBM), solve (HBM only; repeatable on the same inputs), and
 * download (HBM -> host, computational cells / active levels only). */
int sgpu_q_upload(sgpu_context *ctx, const int *ctop, const double *const *dzz, const double *const *dzf,
                  const double *D, const double *const *q, const double *const *src, const double *const *c);
int sgpu_q_solve(sgpu_context *ctx, const sgpu_props *prop, sgpu_stats *stats);
int sgpu_q_download(sgpu_context *ctx, double *const *q);
int sgpu_h_upload(sgpu_context *ctx, const double *D, const double *h, const double *htmp);
int sgpu_h_solve(sgpu_context *ctx, const sgpu_props *prop, sgpu_stats *stats);
int sgpu_h_download(sgpu_context *ctx, double *h);

/* Device-side barrier wait limit in nanoseconds (default 2e9).  A wait that
 * runs out ends the solve with SGPU_TIMEOUT instead of hanging. */
int sgpu_set_timeout_ns(sgpu_context *ctx, long long ns);

/* Device time per barrier-separated phase of the last solve (ns), indexed by
 * phase: pressure solve [1..3] set-up, [4] operator apply, [5] vector update,
 * [6] direction update; free-surface solve [1..2] set-up, [3] apply,
 * [4] update, [5] direction update.  Zero unless the library was built with
 * -DSGPU_PHASE_TIMING. */
int sgpu_phase_times(const sgpu_context *ctx, long long *ns8);

/* Number of CTAs the persistent kernels are launched with (0 = one full wave,
 * the default).  For experiments and tests of the reduction order. */
int sgpu_set_grid(sgpu_context *ctx, int ctas);

/* The CUDA stream (cudaStream_t) every call of this context runs on, so that a
 * caller can order its own work or record timing events around the solves. */
void *sgpu_stream(sgpu_context *ctx);

/* ---------------------------------------------------------------------------
 * Batched mixed-precision pressure solves.
 *
 * Many independent CGSolveQ problems (grids of any size and depth, one
 * qprecond for the batch) share one device arena and advance together in one
 * persistent cooperative kernel; each keeps its own scalars, tolerance and
 * iteration count.  Inner CG arithmetic is FP32; inner products, the solution
 * and the residual used for the stopping test are FP64 ("reliable updates":
 * the FP64 true residual b - A x replaces the FP32 one whenever the iterated
 * residual has fallen by `delta`, and convergence is declared only on it).
 * Same stopping rule as CGSolveQ (main/phys.c:2470-2475, 2516-2524).
 * Type-3 boundary cells are fixed (Dirichlet) values: the CG direction is 0
 * there, so a nonzero src at those cells is not propagated as the reference's
 * p = src does (ComputeQSource never produces one, main/phys.c:2353-2357).
 * No counterpart in the reference (it solves one partition per process).
 * ------------------------------------------------------------------------- */
typedef struct sgpu_batch sgpu_batch;

/* Reserves device memory for up to max_slots cell levels, max_cols
 * computational columns, max_edge_slots edge levels and max_instances
 * problems (sgpu_batch_bytes_per_request gives the bytes one problem needs). */
int sgpu_batch_create(int device, int qprecond, int maxfaces, long long max_slots, long long max_cols,
                      long long max_edge_slots, int max_instances, sgpu_batch **out);
int sgpu_batch_destroy(sgpu_batch *b);
const char *sgpu_batch_last_error(const sgpu_batch *b);
long long sgpu_batch_bytes_per_request(int qprecond, int maxfaces, long long n3, long long ncols,
                                       long long nedge_slots);

/* Adds one problem (same arrays as sgpu_cgsolveq); uploads it and returns its
 * id.  SGPU_OOM when the arena or the instance table is full (admission). */
int sgpu_batch_add(sgpu_batch *b, const sgpu_grid_desc *grid, const int *ctop, const double *const *dzz,
                   const double *const *dzf, const double *D, const double *const *q, const double *const *src,
                   const double *const *c, double qepsilon, int qmaxiters, double resnorm, int *id);

/* One persistent launch: sets up problems added since the last run, then runs
 * up to max_iters global iterations (<= 0: until every problem is done).
 * Reports the problems still running, the device time and the unknown-
 * iterations done in this launch. */
int sgpu_batch_run(sgpu_batch *b, int max_iters, int *running, double *ms, long long *unknown_iters);

/* sgpu_batch_run in two halves, for a host loop that works while the device
 * runs: sgpu_batch_launch enqueues the launch and returns at once; until
 * sgpu_batch_wait, problems may be added and finished problems re-submitted,
 * read back or released (uploads and downloads go on a second stream and touch
 * only problems outside the launch); they join the next launch.
 * sgpu_batch_wait blocks until the launch is done and reports as
 * sgpu_batch_run. */
int sgpu_batch_launch(sgpu_batch *b, int max_iters);
int sgpu_batch_wait(sgpu_batch *b, int *running, double *ms, long long *unknown_iters);

/* State of problem `id` (1 set-up pending, 2 running, 3 done; -1 unknown id). */
int sgpu_batch_state(const sgpu_batch *b, int id);

/* Result and report of a finished problem, scattered into the caller's jagged
 * q (computational cells, levels [ctop, Nk)); q may be NULL for the report
 * only.  release != 0 frees its device memory and id. */
int sgpu_batch_result(sgpu_batch *b, int id, double *const *q, sgpu_stats *stats, int release);

/* Re-submits finished problem `id`.  src (jagged, cell order, as
 * sgpu_batch_add) replaces the right-hand side, or NULL keeps the resident one.
 * warm != 0: the last solution is the initial guess, as phys->qc is for the
 * next CGSolveQ in the model; warm == 0: the initial guess uploaded by
 * sgpu_batch_add is used again.  Grid and coefficients stay resident on the
 * device; only src is uploaded. */
int sgpu_batch_resubmit(sgpu_batch *b, int id, const double *const *src, double qepsilon, int qmaxiters, int warm);

/* Capture each launch sequence (tables in, persistent kernel, report out) in a
 * CUDA graph and replay it while the set of problems is unchanged.  Returns 1
 * when graph launches are in use, 0 when capture is unavailable (direct
 * launches continue).  sgpu_batch_graph_launches counts graph replays. */
int sgpu_batch_use_graph(sgpu_batch *b, int on);
long long sgpu_batch_graph_launches(const sgpu_batch *b);

/* Tuning: reliable-update factor delta (default 0.01), CTA count (0 = full
 * wave), barrier wait limit; pass <= 0 / < 0 to keep a value. */
int sgpu_batch_set(sgpu_batch *b, double delta, int ctas, long long timeout_ns);
/* Tuning: storage slots per tile (4..1024, default 1024) for problems added
 * from now on; a column longer than this still gets a tile of its own.
 * Smaller tiles spread small problems over more CTAs. */
int sgpu_batch_set_tile_slots(sgpu_batch *b, int tile_slots);
/* Tuning: the form of a CG iteration.  1 (default): two passes (operator
 * apply; vector update) with the FP32 solution update x += nu p run in the
 * next apply pass, which streams p anyway (fewer bytes per iteration, a
 * larger pipeline stage); 0: two passes with the update in the vector-update
 * pass -- the same bits as 1.  2 (qprecond 0/1; qprecond 2 runs it as 1): one
 * pass per iteration -- the residual step, the solution update, the new
 * direction and the operator apply in one sweep with one grid barrier, the
 * next mu from the sweep's own inner products (|r - nu z|^2 = r.r - 2 nu r.z
 * + nu^2 z.z); the same stopping rule on the FP64 true residual, iterates
 * that round differently.  Refused while a problem is in mid-solve under
 * another form.  (A tuning knob of this engine; the reference has none.) */
int sgpu_batch_set_fusion(sgpu_batch *b, int form);
/* Scheduling: problem `id` advances only on the global iterations it of a
 * launch with it % stride == 0 (1, the default: on every one; 1..64).  Every
 * global iteration costs time in proportion to the work of the problems that
 * take part, so giving large problems a stride > 1 while small ones are in
 * flight lets the small ones finish sooner.  A problem's own iterates, and so
 * its result bits and iteration count, do not depend on its stride.  May be
 * changed between launches, also in mid-solve.  (A scheduling knob of this
 * engine; the reference has none.) */
int sgpu_batch_set_stride(sgpu_batch *b, int id, int stride);
void *sgpu_batch_stream(sgpu_batch *b);

/* Device time of the last launch per phase (ns): [1] operator apply, [2]
 * vector update, [3] FP64 merge, [4] FP64 true residual, [5..7] set-up.
 * Zero unless the library was built with -DSGPU_PHASE_TIMING. */
int sgpu_batch_phase_times(const sgpu_batch *b, long long *ns8);

/* Grid of sgpu_cgsolve_noalloc: the same gridT fields as sgpu_grid_desc, but
 * every pointer is DEVICE memory owned by the caller, in the caller's cell
 * order (no reordering, no copies). */
typedef struct sgpu_noalloc_grid {
  int Nc, Ne, maxfaces;
  int ncomp;           /* celldist[1]: cellp[0..ncomp) are the computational cells */
  const int *cellp;    /* device [ncomp]                                          */
  const int *nfaces;   /* device [Nc]                                              */
  const int *neigh;    /* device [Nc*maxfaces], -1 = no neighbour                  */
  const int *face;     /* device [Nc*maxfaces]                                     */
  const double *Ac;    /* device [Nc]                                              */
  const double *df;    /* device [Ne]                                              */
  const double *dg;    /* device [Ne]                                              */
} sgpu_noalloc_grid;

/* Free-surface solve (the CGSolve semantics above) that allocates nothing.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- a host program whose device memory is owned entirely by its own
 * pool allocator (a coupled model that hands each component slices of one
 * arena and forbids other allocations), or a time-critical loop that cannot
 * pay for cudaMalloc/cudaFree, which synchronise the whole device.
 *   D, htmp   device inputs [Ne], [Nc];  h  device [Nc], type-3 values in,
 *             solution out at computational cells (in place, as CGSolve does);
 *   stream    the cudaStream_t to run on (0 = legacy default stream).
 * The solver's scratch is one static device array of 32 MiB in this library:
 * 512 + 16*2048 + 8*Nc*(5+maxfaces) bytes must fit, i.e. up to about 466,000
 * quadrilateral or 524,000 triangular cells; larger grids return
 * SGPU_TOO_LARGE before any device work.  Every call shares that array and
 * leaves its contents behind (the control words are cleared at the start of
 * each call), so calls that overlap on the GPU race and must not be issued.
 * The first call on each device looks up the array's address
 * (cudaGetSymbolAddress, with that device current); make it before any stream
 * capture.  The address is kept per device and context, so the first call
 * after a cudaDeviceReset looks it up again (also before any capture).  Runs on the current device; blocks until the solve has finished.
 * stats->ms_solve is -1 (no timing events are created). */
int sgpu_cgsolve_noalloc(const sgpu_noalloc_grid *grid, const double *D, double *h, const double *htmp,
                         const sgpu_props *prop, sgpu_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif
#endif
