// sgpu_q.cu -- the nonhydrostatic pressure PCG (CGSolveQ) as one persistent,
// cooperative kernel per solve, FP64 throughout.
//
// Reference semantics followed (main/phys.c of SUNTANS):
//   CGSolveQ        2411-2550  the solve: setup, initial residual, loop, rescale
//   OperatorQ       3486-3536  y = A x  (qprecond 0 and 2)
//   OperatorQC      3364-3409  y = C^-1 A C^-1 x with unit diagonal (qprecond 1)
//   QCoefficients   3420-3471  vertical coef, and fcoef for qprecond 1
//   ConditionQ      3629-3687  c = sqrt(|diag A|) (qprecond 1)
//   Preconditioner  3577-3619  per-column tridiagonal solve (qprecond 2)
//   TriSolve        util.c:185-203
//   InnerProduct3   3304-3319  sum over computational cells, k in [ctop, Nk)
//
// Data layout (device order): column j = cellp[j] for j < ncomp (computational
// cells), then the type-3 boundary cells, then any remaining cells.  Column j
// holds levels [0, Nk) at [dcoff[j], dcoff[j+1]).  Slots k < ctop (dry layers)
// are kept at 0 in every working vector, so vector phases run over the whole
// computational storage [0, n3c) without masks.  Face coefficients are F
// separate arrays fc[f][u] over the computational storage (0 where the face
// does not couple that level).
//
// Work split: computational columns are packed into tiles of at most 512
// storage slots; a CTA of 256 threads owns tiles b, b+G, b+2G, ... in every
// phase, 2 slots per thread.  Barriers: 3 per CG iteration, each finalised by
// the last CTA to arrive (deterministic reduction, scalar recurrences).
#include "sgpu_common.cuh"
#include "sgpu_q.h"

// unroll factor of the flat apply loop (slots of one thread in flight together)
#ifndef SGPU_Q_UNROLL
#define SGPU_Q_UNROLL 1
#endif
#define SGPU_Q_PRAGMA(x) _Pragma(#x)
#define SGPU_Q_UNROLL_N(n) SGPU_Q_PRAGMA(unroll n)
#define SGPU_Q_APPLY_UNROLL SGPU_Q_UNROLL_N(SGPU_Q_UNROLL)
#ifndef SGPU_Q_MINB
#define SGPU_Q_MINB 6
#endif

namespace sgpu {

struct TileCtx {
  int base;      // storage offset of the tile's first slot
  int len;       // slots in the tile
  int c0;        // first column
  int ncols;     // columns in the tile
};

__device__ __forceinline__ void tile_load(const QArgs& a, int t, TileCtx& tc, int* s_start) {
  const int c0 = a.tile_col[t];
  const int c1 = a.tile_col[t + 1];
  const int base = a.dcoff[c0];
  for (int c = threadIdx.x; c <= c1 - c0; c += kBlock) s_start[c] = a.dcoff[c0 + c] - base;
  tc.base = base;
  tc.c0 = c0;
  tc.ncols = c1 - c0;
  tc.len = a.dcoff[c1] - base;
  __syncthreads();
}

// column (local index) holding local slot s: largest c with s_start[c] <= s
__device__ __forceinline__ int find_col(const int* s_start, int ncols, int s) {
  int lo = 0, hi = ncols - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (s_start[mid] <= s) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// operator apply for one slot u = (column j, level k), k in [ctop, Nk)
// ---------------------------------------------------------------------------
template <int QP>
__device__ __forceinline__ double apply_slot(const QArgs& a, const double* __restrict__ xin, int u, int j, int k,
                                             int ctop, int nk) {
  const int F = a.F;
  double y;
  if (QP == 1) {
    // OperatorQC: y = -x + sum_f fcoef*x[nc] + vertical neighbours (3364-3409)
    y = -xin[u];
    for (int f = 0; f < F; ++f) {
      const int meta = a.fmeta[j * F + f];
      if (meta < 0) continue;
      const int kmin = meta & 0xffff, kmax = meta >> 16;
      if (k >= kmin && k < kmax) y += xin[a.fnoff[j * F + f] + k] * a.fc[(size_t)f * a.n3c + u];
    }
    if (k > ctop && k < nk - 1) {
      // the two vertical terms as two FMAs into y (GB300's FP64 pipe is the
      // kernel's limit: a product, an FMA and an add would be three)
      y = __fma_rn(a.coef[u], xin[u - 1], y);
      y = __fma_rn(a.coef[u + 1], xin[u + 1], y);
    } else if (ctop < nk - 1) {
      if (k == ctop) y += a.coef[u + 1] * xin[u + 1];
      else y += a.coef[u] * xin[u - 1];  // k == nk-1
    }
  } else {
    // OperatorQ: horizontal differences then vertical (3486-3536)
    const double xu = xin[u];
    y = 0.0;
    for (int f = 0; f < F; ++f) {
      const int meta = a.fmeta[j * F + f];
      if (meta < 0) continue;
      const int kmin = meta & 0xffff, kmax = meta >> 16;
      if (k >= kmin && k < kmax) y += (xin[a.fnoff[j * F + f] + k] - xu) * a.fc[(size_t)f * a.n3c + u];
    }
    if (ctop < nk - 1) {
      if (k == ctop) {
        const double c0 = a.coef[u], c1 = a.coef[u + 1];
        y += (-2 * c0 - c1) * xu + c1 * xin[u + 1];
      } else if (k == nk - 1) {
        const double c0 = a.coef[u];
        y += c0 * xin[u - 1] - c0 * xu;
      } else {
        const double c0 = a.coef[u], c1 = a.coef[u + 1];
        y += c0 * xin[u - 1] - (c0 + c1) * xu + c1 * xin[u + 1];
      }
    } else {
      y -= 2.0 * a.coef[u] * xu;
    }
  }
  return y;
}

// Branch-free form of apply_slot for the loop's flat apply: every load of a
// slot is issued unconditionally (a face that does not couple the level reads
// the slot itself and has coefficient fc = 0; vertical neighbours outside the
// column get coefficient 0), so the loads of several slots overlap.  The sums
// are those of apply_slot: terms with a zero coefficient add exactly 0.
// Dry slots (k < ctop) return 0.  FF: compile-time face count (0 = a.F).
template <int QP, int FF>
__device__ __forceinline__ double apply_flat(const QArgs& a, const double* __restrict__ xin, int u) {
  const int F = FF ? FF : a.F;
  // the slot's wet / upper / lower-neighbour bits (set-up S1): no column lookup
  const int fl = a.sflag[u];
  const bool act = fl & 1, up = fl & 2, dn = fl & 4;
  const double xu = xin[u];
  double y = (QP == 1) ? -xu : 0.0;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    // the neighbour slot comes straight from the slot (set-up S1), so the
    // gather waits on one load, not on the slot's column metadata first
    const int n = a.nslot[(size_t)f * a.n3c + u];
    const double w = a.fc[(size_t)f * a.n3c + u];
    if (QP == 1) y = __fma_rn(xin[n], w, y);
    else y = __fma_rn(xin[n] - xu, w, y);
  }
  const double xm = xin[u > 0 ? u - 1 : 0], xp = xin[u + 1];
  const double c0 = a.coef[u], c1 = a.coef[u + 1];
  if (QP == 1) {
    const double cm = up ? c0 : 0.0;
    const double cp = dn ? c1 : 0.0;
    y = __fma_rn(cm, xm, y);  // two FMAs, as in apply_slot
    y = __fma_rn(cp, xp, y);
  } else if (up || dn) {  // ctop < nk - 1
    if (!up) y += (-2 * c0 - c1) * xu + c1 * xp;  // k == ctop
    else if (!dn) y += c0 * xm - c0 * xu;         // k == nk - 1
    else y += c0 * xm - (c0 + c1) * xu + c1 * xp;
  } else {
    y -= 2.0 * c0 * xu;
  }
  return act ? y : 0.0;
}

// Thomas solve of one column with the factors prepared at setup:
//   d'[k] = d[k] - w[k] d'[k-1];  u[k] = (d'[k] - cup[k] u[k+1]) * ib[k]
// cup[k] = coef[k+1] (the reference's c[k], 3589-3597).  Single-level column:
// u = -0.5 d / coef (3617).
__device__ __forceinline__ void column_solve(const QArgs& a, const double* rin, double* out, int off, int ctop,
                                             int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) {
    out[b] = -0.5 * rin[b] / a.coef[b];
    return;
  }
  double dprev = rin[b];
  out[b] = dprev;
  for (int u = b + 1; u < e; ++u) {
    dprev = rin[u] - a.tw[u] * dprev;
    out[u] = dprev;
  }
  double unext = out[e - 1] * a.tib[e - 1];
  out[e - 1] = unext;
  for (int u = e - 2; u >= b; --u) {
    unext = (out[u] - a.coef[u + 1] * unext) * a.tib[u];
    out[u] = unext;
  }
}

// Staged tile of the qprecond-2 vector update: r, the Thomas factors, the
// vertical coefficients (one past the tile) and the solve's output.
struct TriSmem {
  double r[kTileCap], w[kTileCap], ib[kTileCap], cf[kTileCap + 1], out[kTileCap];
};

// column_solve on a staged tile: the column's slots start at local offset off.
__device__ __forceinline__ void column_solve_smem(TriSmem& sm, int off, int ctop, int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) {
    sm.out[b] = -0.5 * sm.r[b] / sm.cf[b];
    return;
  }
  double dprev = sm.r[b];
  sm.out[b] = dprev;
  for (int u = b + 1; u < e; ++u) {
    dprev = sm.r[u] - sm.w[u] * dprev;
    sm.out[u] = dprev;
  }
  double unext = sm.out[e - 1] * sm.ib[e - 1];
  sm.out[e - 1] = unext;
  for (int u = e - 2; u >= b; --u) {
    unext = (sm.out[u] - sm.cf[u + 1] * unext) * sm.ib[u];
    sm.out[u] = unext;
  }
}

// Factorisation of one column for column_solve (TriSolve's forward sweep on b,
// util.c:191-195): b'[0]=b[0], b'[k]=b[k]-a[k]*c[k-1]/b'[k-1]; w[k]=a[k]/b'[k-1]; ib=1/b'.
__device__ __forceinline__ void column_factor(const QArgs& a, int off, int ctop, int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) return;
  double bp = -2 * a.coef[b] - a.coef[b + 1];
  a.tib[b] = 1.0 / bp;
  for (int u = b + 1; u < e; ++u) {
    const double ak = a.coef[u];
    const double ck1 = a.coef[u];  // c[k-1] = coef[k]
    const double bk = (u == e - 1) ? -a.coef[u] : (-a.coef[u] - a.coef[u + 1]);
    const double bnew = bk - ak * ck1 / bp;
    a.tw[u] = ak / bp;
    bp = bnew;
    a.tib[u] = 1.0 / bp;
  }
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
template <int QP>
__global__ void __launch_bounds__(kBlock, SGPU_Q_MINB) cgsolveq_kernel(QArgs a) {
  __shared__ int s_start[kMaxTileCols + 1];
  __shared__ double s_red[2 * kBlock + 2];
  __shared__ double s_sc[4];  // scalars from thread 0: mu, nu, done
  __shared__ TriSmem s_tri;
  SolveCtl* ctl = a.ctl;
  const int G = gridDim.x;
  const int F = a.F;
  const int tid = threadIdx.x;
  // Barriers: arrive-and-wait on a monotonic counter; after each, one warp of
  // every CTA sums the published per-CTA partials in the same order and
  // thread 0 runs the scalar recurrences (identical in every CTA), leaving
  // mu, nu and the loop flag in shared memory.  Partials rotate between two
  // buffers so that no CTA overwrites a set another is still reading.
  unsigned int nbar = 0;
  double* partA = a.partials;          // [2][G]: p.z
  double* partB = a.partials + 2 * G;  // [2][2][G]: r.r or r.s, r.r

  // ---- S1: working vectors, face metadata, coefficients / conditioner ----
  for (int t = blockIdx.x; t < a.ntiles; t += G) {
    TileCtx tc;
    tile_load(a, t, tc, s_start);
    for (int s = tid; s < tc.len; s += kBlock) {
      const int cl = find_col(s_start, tc.ncols, s);
      const int j = tc.c0 + cl;
      const int k = s - s_start[cl];
      const int u = tc.base + s;
      const int ctop = a.ctop[j];
      const int nk = a.nk[j];
      const bool act = k >= ctop;
      a.sflag[u] = (unsigned char)((act ? 1 : 0) | (act && k > ctop ? 2 : 0) | (act && k < nk - 1 ? 4 : 0));
      a.z[u] = 0.0;
      a.r[u] = 0.0;
      a.rt[u] = 0.0;
      double diag = 0.0;
      for (int f = 0; f < F; ++f) {
        const int nb = a.nbr[j * F + f];
        int kmin = 0, kmax = 0, meta = -1;
        if (nb >= 0) {
          const int e = a.fedge[j * F + f];
          kmin = max(ctop, a.ctop[nb]);
          kmax = a.nke[e];
          meta = kmin | (kmax << 16);
          if (k == 0) {
            a.fmeta[j * F + f] = meta;
            a.fnoff[j * F + f] = a.dcoff[nb];
          }
          const bool on = act && k >= kmin && k < kmax;
          a.nslot[(size_t)f * a.n3c + u] = on ? a.dcoff[nb] + k : u;
          if (QP != 1) {
            a.fc[(size_t)f * a.n3c + u] = on ? a.dzf[a.eoff[e] + k] * a.D[e] : 0.0;
          } else {
            if (on) diag += a.dzz[u] * a.D[e];
            a.fc[(size_t)f * a.n3c + u] = 0.0;
          }
        } else {
          if (k == 0) {
            a.fmeta[j * F + f] = -1;
            a.fnoff[j * F + f] = 0;
          }
          a.nslot[(size_t)f * a.n3c + u] = u;
          a.fc[(size_t)f * a.n3c + u] = 0.0;
        }
      }
      const double Ac = a.Ac[j];
      if (QP != 1) {
        // QCoefficients, qprecond != 1 branch (3459-3468)
        double cf = 0.0;
        if (k == ctop) cf = Ac / a.dzz[u];
        else if (k > ctop) cf = 2 * Ac / (a.dzz[u] + a.dzz[u - 1]);
        a.coef[u] = cf;
        a.x[u] = act ? a.q_in[u] : 0.0;
        a.p[u] = act ? a.src_in[u] : 0.0;
      } else {
        // ConditionQ vertical part (3660-3675) and sqrt (3678-3685)
        if (act) {
          const double ak = (k == ctop) ? Ac / a.dzz[u] : 2 * Ac / (a.dzz[u] + a.dzz[u - 1]);
          if (ctop < nk - 1) {
            if (k == ctop) {
              const double ak1 = 2 * Ac / (a.dzz[u + 1] + a.dzz[u]);
              diag += 2 * ak + ak1;
            } else if (k == nk - 1) {
              diag += ak;
            } else {
              const double ak1 = 2 * Ac / (a.dzz[u + 1] + a.dzz[u]);
              diag += (ak + ak1);
            }
          }
          if (diag <= 0) diag = 1;
          const double cu = sqrt(diag);
          a.c[u] = cu;
          a.p[u] = a.src_in[u] / cu;
          a.x[u] = a.q_in[u] * cu;
        } else {
          a.c[u] = 1.0;
          a.p[u] = 0.0;
          a.x[u] = 0.0;
        }
        a.coef[u] = 0.0;
      }
    }
    if (QP == 2) {
      __syncthreads();
      for (int cl = tid; cl < tc.ncols; cl += kBlock) {
        const int j = tc.c0 + cl;
        column_factor(a, tc.base + s_start[cl], a.ctop[j], a.nk[j]);
      }
    }
    __syncthreads();
  }
  // boundary / remaining columns: given values, never updated (read as neighbours)
  for (int u = a.n3c + blockIdx.x * kBlock + tid; u < a.n3; u += G * kBlock) {
    a.x[u] = a.q_in[u];
    a.p[u] = a.src_in[u];
    if (QP == 1) a.c[u] = a.c_in[u];
  }
  if (!grid_wait(ctl, ++nbar * G, 1)) return;

  // ---- S2 (qprecond 1): scaled coefficients (QCoefficients 3427-3452) ----
  if (QP == 1) {
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      TileCtx tc;
      tile_load(a, t, tc, s_start);
      for (int s = tid; s < tc.len; s += kBlock) {
        const int cl = find_col(s_start, tc.ncols, s);
        const int j = tc.c0 + cl;
        const int k = s - s_start[cl];
        const int u = tc.base + s;
        const int ctop = a.ctop[j];
        if (k < ctop) continue;
        const double Ac = a.Ac[j];
        if (k == ctop) a.coef[u] = Ac / a.dzz[u] / a.c[u];
        else a.coef[u] = 2 * Ac / (a.dzz[u] + a.dzz[u - 1]) / (a.c[u] * a.c[u - 1]);
        for (int f = 0; f < F; ++f) {
          const int meta = a.fmeta[j * F + f];
          if (meta < 0) continue;
          const int kmin = meta & 0xffff, kmax = meta >> 16;
          if (k >= kmin && k < kmax) {
            const int e = a.fedge[j * F + f];
            a.fc[(size_t)f * a.n3c + u] = a.dzz[u] * a.D[e] / (a.c[u] * a.c[a.fnoff[j * F + f] + k]);
          }
        }
      }
      __syncthreads();
    }
    if (!grid_wait(ctl, ++nbar * G, 2)) return;
  }

  // ---- S3: z = A x; r = p - z; p = r or M^-1 r; alpha0, eps0 (2444-2475) ----
  // thread 0 of every CTA keeps the scalar state (the same in every CTA)
  double alpha = 0.0, eps = 0.0, eps0 = 0.0, mu_t = 0.0;
  int status = SGPU_OK;
  {
    double part[2] = {0.0, 0.0};
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      TileCtx tc;
      tile_load(a, t, tc, s_start);
      for (int s = tid; s < tc.len; s += kBlock) {
        const int cl = find_col(s_start, tc.ncols, s);
        const int j = tc.c0 + cl;
        const int k = s - s_start[cl];
        const int u = tc.base + s;
        const int ctop = a.ctop[j];
        if (k < ctop) continue;
        const double zu = apply_slot<QP>(a, a.x, u, j, k, ctop, a.nk[j]);
        a.z[u] = zu;
        const double ru = a.p[u] - zu;
        a.r[u] = ru;
        if (QP != 2) {
          a.p[u] = ru;
          part[0] += ru * ru;
        }
      }
      if (QP == 2) {
        __syncthreads();
        for (int cl = tid; cl < tc.ncols; cl += kBlock) {
          const int j = tc.c0 + cl;
          column_solve(a, a.r, a.rt, tc.base + s_start[cl], a.ctop[j], a.nk[j]);
        }
        __syncthreads();
        for (int s = tid; s < tc.len; s += kBlock) {
          const int u = tc.base + s;
          const double ru = a.r[u], rtu = a.rt[u];
          a.p[u] = rtu;
          part[0] += ru * rtu;
          part[1] += ru * ru;
        }
      }
      __syncthreads();
    }
    cta_sum<2, kBlock>(part, s_red);
    if (tid == 0) {
      partB[2 * G + blockIdx.x] = part[0];
      partB[3 * G + blockIdx.x] = part[1];
    }
    if (!grid_wait(ctl, ++nbar * G, 3)) return;
    grid_sum<2>(partB + 2 * G, G, [&](const double* tot) {
      alpha = tot[0];
      double alpha0 = tot[0];
      if (!a.resnorm) alpha0 = 1;
      if (QP == 2) eps = eps0 = tot[1];
      else eps = eps0 = alpha0;
      s_sc[0] = 0.0;
      s_sc[1] = 0.0;
      s_sc[2] = (a.maxiters <= 0 || eps == 0) ? 1.0 : 0.0;
    });
  }

  // ---- the CG loop (2478-2525) ----
  // Every update and inner-product term is one explicit FMA: the loop is
  // bound by GB300's FP64 pipe, and a product and a sum issued apart would
  // cost two of its slots.
  // x += nu p (2506-2507) is carried out in C, where p is read anyway, before
  // p changes: the same operation on the same operands, one read and one
  // write of p fewer per iteration.  When the loop ends after B, the last one
  // is still pending and is done at the end.
  bool x_pending = false;
  int n = 0;
  for (;;) {
    if (s_sc[2] != 0.0) break;
    // A: z = A p, p.z -- flat over the computational storage: slot u of
    // thread g is u = g + i*T (T = all threads), its column from the static
    // slot-to-column index, so no tile barrier or column search stands between
    // a slot's loads and the next slot's.
    {
      double part[1] = {0.0};
      const int T = G * kBlock;
      if (F == 3) {
SGPU_Q_APPLY_UNROLL
        for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += T) {
          const double zu = apply_flat<QP, 3>(a, a.p, u);
          a.z[u] = zu;
          part[0] = __fma_rn(a.p[u], zu, part[0]);
        }
      } else if (F == 4) {
SGPU_Q_APPLY_UNROLL
        for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += T) {
          const double zu = apply_flat<QP, 4>(a, a.p, u);
          a.z[u] = zu;
          part[0] = __fma_rn(a.p[u], zu, part[0]);
        }
      } else {
        for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += T) {
          const double zu = apply_flat<QP, 0>(a, a.p, u);
          a.z[u] = zu;
          part[0] = __fma_rn(a.p[u], zu, part[0]);
        }
      }
      cta_sum<1, kBlock>(part, s_red);
      if (tid == 0) partA[(n & 1) * G + blockIdx.x] = part[0];
      if (!grid_wait(ctl, ++nbar * G, 4)) return;
      grid_sum<1>(partA + (n & 1) * G, G, [&](const double* tot) {
        mu_t = 1 / alpha;
        const double nu = alpha / tot[0];
        s_sc[1] = nu;
        if (!isfinite(nu)) {
          status = SGPU_BREAKDOWN;
          s_sc[2] = 1.0;
        }
      });
      if (s_sc[2] != 0.0) break;
    }
    // B: r -= nu z; [rt = M^-1 r]; alpha, eps
    {
      const double nu = s_sc[1];
      double part[2] = {0.0, 0.0};
      if (QP != 2) {
        const int T = G * kBlock;
#pragma unroll 4
        for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += T) {
          const double ru = __fma_rn(-nu, a.z[u], a.r[u]);
          a.r[u] = ru;
          part[0] = __fma_rn(ru, ru, part[0]);
        }
      }
      // qprecond 2: the tile's r, Thomas factors and coefficients are staged
      // in shared memory and each column is solved there (one thread per
      // column), then M^-1 r leaves coalesced.
      for (int t = blockIdx.x; QP == 2 && t < a.ntiles; t += G) {
        const int c0 = a.tile_col[t], c1 = a.tile_col[t + 1];
        const int base = a.dcoff[c0], end = a.dcoff[c1], len = end - base;
        for (int sl = tid; sl <= len; sl += kBlock) {
          const int u = base + sl;
          if (sl < len) {
            const double ru = a.r[u] - nu * a.z[u];
            a.r[u] = ru;
            s_tri.r[sl] = ru;
            s_tri.w[sl] = a.tw[u];
            s_tri.ib[sl] = a.tib[u];
            s_tri.out[sl] = 0.0;  // dry levels (k < ctop) are not solved and stay 0
          }
          s_tri.cf[sl] = a.coef[u];
        }
        for (int c = tid; c <= c1 - c0; c += kBlock) s_start[c] = a.dcoff[c0 + c] - base;
        __syncthreads();
        for (int c = tid; c < c1 - c0; c += kBlock)
          column_solve_smem(s_tri, s_start[c], a.ctop[c0 + c], a.nk[c0 + c]);
        __syncthreads();
        for (int sl = tid; sl < len; sl += kBlock) {
          const double ru = s_tri.r[sl], rtu = s_tri.out[sl];
          a.rt[base + sl] = rtu;
          part[0] += ru * rtu;
          part[1] += ru * ru;
        }
        __syncthreads();
      }
      cta_sum<2, kBlock>(part, s_red);
      if (tid == 0) {
        partB[(size_t)(n & 1) * 2 * G + blockIdx.x] = part[0];
        partB[(size_t)(n & 1) * 2 * G + G + blockIdx.x] = part[1];
      }
      if (!grid_wait(ctl, ++nbar * G, 5)) return;
      grid_sum<2>(partB + (size_t)(n & 1) * 2 * G, G, [&](const double* tot) {
        alpha = tot[0];
        mu_t *= alpha;
        s_sc[0] = mu_t;
        eps = (QP == 2) ? tot[1] : alpha;
        const bool conv = sqrt(eps / eps0) < a.qepsilon;
        double done = 0.0;
        if (conv || eps == 0) done = 1.0;
        else if (n + 1 >= a.maxiters) {
          status = SGPU_MAXITER;
          done = 1.0;
        }
        if (!isfinite(alpha)) {
          status = SGPU_BREAKDOWN;
          done = 1.0;
        }
        s_sc[2] = done;
      });
      x_pending = true;
      ++n;
      if (s_sc[2] != 0.0) break;
    }
    // C: x += nu p; p = r + mu p  (or rt + mu p)
    {
      const double mu = s_sc[0];
      const double nu = s_sc[1];
      const double* src = (QP == 2) ? a.rt : a.r;
      const int T = G * kBlock;
#pragma unroll 4
      for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += T) {
        const double pu = a.p[u];
        a.x[u] = __fma_rn(nu, pu, a.x[u]);
        a.p[u] = __fma_rn(mu, pu, src[u]);
      }
      x_pending = false;
      if (!grid_wait(ctl, ++nbar * G, 6)) return;
    }
  }
  const double nu_last = s_sc[1];
  if (blockIdx.x == 0 && tid == 0) {
    ctl->alpha = alpha;
    ctl->eps = eps;
    ctl->eps0 = eps0;
    ctl->mu = mu_t;
    ctl->nu = nu_last;
    ctl->n = n;
    if (status != SGPU_OK) atomicCAS(&ctl->status, SGPU_OK, status);
    ctl->done = 1;
  }

  // ---- the pending x update, and the rescale (2539-2546), each slot by one thread ----
  if (QP == 1) {
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int base = a.dcoff[a.tile_col[t]], end = a.dcoff[a.tile_col[t + 1]];
      for (int u = base + tid; u < end; u += kBlock) {
        if (x_pending) a.x[u] += nu_last * a.p[u];
        a.x[u] /= a.c[u];
      }
    }
  } else if (x_pending) {
    for (int u = blockIdx.x * kBlock + tid; u < a.n3c; u += G * kBlock) a.x[u] += nu_last * a.p[u];
  }
}

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------
template <int QP>
static cudaError_t launch_q(const QArgs& a, int grid, cudaStream_t st) {
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)cgsolveq_kernel<QP>, dim3(grid), dim3(kBlock), args, 0, st);
}

int q_max_grid(int qprecond, int device) {
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const void* fn = qprecond == 1 ? (const void*)cgsolveq_kernel<1>
                 : qprecond == 2 ? (const void*)cgsolveq_kernel<2> : (const void*)cgsolveq_kernel<0>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kBlock, 0) != cudaSuccess) return 0;
  return sms * per;
}

cudaError_t q_launch(const QArgs& a, int qprecond, int grid, cudaStream_t st) {
  switch (qprecond) {
    case 0: return launch_q<0>(a, grid, st);
    case 1: return launch_q<1>(a, grid, st);
    case 2: return launch_q<2>(a, grid, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace sgpu
