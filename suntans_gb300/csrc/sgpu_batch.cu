// sgpu_batch.cu -- batched, mixed-precision pressure solver (CGSolveQ
// semantics, main/phys.c:2411-2550) for many independent grids in one
// persistent cooperative launch.
//
// Precision scheme ("reliable updates", a defect-correction form of CG):
//   * the CG iteration runs on FP32 vectors: operator apply, preconditioner
//     (Jacobi through the scaling of qprecond 1, the column tridiagonal solve of
//     qprecond 2), and the vector updates;
//   * every inner product (p.Ap, r.r, r.M^-1 r) is accumulated in FP64 from
//     exact products of FP32 values (a product of two floats is exact in FP64);
//   * the solution is accumulated in FP64: the FP32 increments collected since
//     the last update are added into the FP64 iterate whenever the iterated
//     residual norm has fallen by delta (default 0.01) since the last update, and
//     the TRUE residual b - A x is then recomputed in FP64 with FP64
//     coefficients and replaces the FP32 residual (the Krylov direction p is
//     kept, so no convergence is lost).  Convergence is declared only on that
//     FP64 true residual: sqrt(eps/eps0) < qepsilon with the reference's own eps
//     and eps0 (main/phys.c:2470-2475, 2516-2524).
//
// The operators are the reference's: OperatorQC (3364-3409) with the
// coefficients of QCoefficients/ConditionQ (3420-3471, 3629-3687) for
// qprecond 1, OperatorQ (3486-3536) for qprecond 0 and 2, Preconditioner +
// TriSolve (3577-3619, util.c:185-203) for qprecond 2.  In the FP32 apply the
// qprecond 1 face and vertical coefficients are formed on the fly from dzz and
// 1/c (2 floats per level instead of F+1), and the qprecond 0/2 face
// coefficients dzf*D are read from edge storage (each edge level serves both
// of its cells).
//
// Per global iteration: phase A (p_new = s + mu p_old formed on the fly for the
// cell and its neighbours, z = A p_new, p.z), phase B (x += nu p, r -= nu z,
// preconditioner, r.s and r.r), and, only when some instance asked for it, the
// reliable-update phases R1 (x64 += x32) and R2 (FP64 true residual).  Each
// phase ends at a grid barrier; the per-instance reductions finish before it
// in the CTA that completes the instance's last tile.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/suntans_gb300.h"
#include "sgpu_batch.h"

namespace sgpu {

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f2d(float f) { return (double)f; }

struct TileInfo {
  int c0, c1;     // global columns [c0, c1)
  int base, end;  // storage slots [base, end)
  int inst;
};

__device__ __forceinline__ void load_tile(const BatchArgs& a, int t, TileInfo& ti, int* s_start, int* s_ctop,
                                          int* s_nk) {
  const int c0 = a.tile_c0[2 * t], c1 = a.tile_c0[2 * t + 1];
  ti.c0 = c0;
  ti.c1 = c1;
  ti.inst = a.tile_inst[t];
  const int base = a.col[c0].s;
  ti.base = base;
  for (int c = threadIdx.x; c < c1 - c0; c += blockDim.x) {
    const BCol cc = a.col[c0 + c];
    s_start[c] = cc.s - base;
    s_ctop[c] = cc.ctop;
    s_nk[c] = cc.nk;
  }
  if (threadIdx.x == 0) {
    const BCol cl = a.col[c1 - 1];
    s_start[c1 - c0] = cl.s + cl.nk - base;
  }
  __syncthreads();
  ti.end = base + s_start[c1 - c0];
}

__device__ __forceinline__ int find_col_b(const int* s_start, int ncols, int s) {
  int lo = 0, hi = ncols - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (s_start[mid] <= s) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Deterministic per-instance reduction: the CTA that finishes the last tile of
// instance `i` in this phase sums the tiles' partials in tile order and runs
// `fin(tot)` on thread 0.  Must be called by the whole CTA after block_sum.
template <int NV, class Fin>
__device__ __forceinline__ void tile_done(const BatchArgs& a, int t, int i, const double (&part)[NV], double* s_red,
                                          Fin&& fin) {
  __shared__ int s_last;
  BInst* I = a.inst + i;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) a.tpart[2 * t + v] = part[v];
    __threadfence();
    const int old = atomicAdd(&I->cnt, 1);
    s_last = (old == I->t1 - I->t0 - 1);
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    double v[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int tt = I->t0 + (int)threadIdx.x; tt < I->t1; tt += blockDim.x)
        s += ((volatile double*)a.tpart)[2 * tt + j];
      v[j] = s;
    }
    block_sum<NV>(v, s_red);
    if (threadIdx.x == 0) {
      fin(I, v);
      I->cnt = 0;
      __threadfence();
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int inst_state(const BatchArgs& a, int i) { return ld_volatile_int(&a.inst[i].state); }
__device__ __forceinline__ int inst_flags(const BatchArgs& a, int i) { return ld_volatile_int(&a.inst[i].flags); }

// ---- FP64 operator (true residual), one active slot ----
template <int QP>
__device__ __forceinline__ double apply64(const BatchArgs& a, int u, int j, int k, int ctop, int nk, const double* x) {
  const int F = a.F;
  double y;
  if (QP == 1) {
    y = -x[u];
    for (int f = 0; f < F; ++f) {
      const BFace fc = a.face[(size_t)j * F + f];
      if (fc.ns < 0 || k < fc.kmin || k >= fc.kmax) continue;
      y += x[fc.ns + k] * a.fc64[(size_t)F * u + f];
    }
    if (k > ctop) y += a.coef64[u] * x[u - 1];
    if (k < nk - 1) y += a.coef64[u + 1] * x[u + 1];
  } else {
    const double xu = x[u];
    y = 0.0;
    for (int f = 0; f < F; ++f) {
      const BFace fc = a.face[(size_t)j * F + f];
      if (fc.ns < 0 || k < fc.kmin || k >= fc.kmax) continue;
      y += (x[fc.ns + k] - xu) * a.dzfD64[fc.es + k];
    }
    if (ctop < nk - 1) {
      if (k == ctop) {
        const double c0 = a.coef64[u], c1 = a.coef64[u + 1];
        y += (-2 * c0 - c1) * xu + c1 * x[u + 1];
      } else if (k == nk - 1) {
        const double c0 = a.coef64[u];
        y += c0 * x[u - 1] - c0 * xu;
      } else {
        const double c0 = a.coef64[u], c1 = a.coef64[u + 1];
        y += c0 * x[u - 1] - (c0 + c1) * xu + c1 * x[u + 1];
      }
    } else {
      y -= 2.0 * a.coef64[u] * xu;
    }
  }
  return y;
}

// FP32 Thomas solve of one column with FP32 factors (qprecond 2).
__device__ __forceinline__ void column_solve32(const BatchArgs& a, int off, int ctop, int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) {
    a.s32[b] = -0.5f * a.r32[b] / a.coef32[b];
    return;
  }
  float dprev = a.r32[b];
  a.s32[b] = dprev;
  for (int u = b + 1; u < e; ++u) {
    dprev = __fmaf_rn(-a.tw32[u], dprev, a.r32[u]);
    a.s32[u] = dprev;
  }
  float un = a.s32[e - 1] * a.tib32[e - 1];
  a.s32[e - 1] = un;
  for (int u = e - 2; u >= b; --u) {
    un = __fmaf_rn(-a.coef32[u + 1], un, a.s32[u]) * a.tib32[u];
    a.s32[u] = un;
  }
}

// FP64 factorisation of one column (TriSolve's forward sweep), stored in FP32.
__device__ __forceinline__ void column_factor64(const BatchArgs& a, int off, int ctop, int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) return;
  double bp = -2 * a.coef64[b] - a.coef64[b + 1];
  a.tib32[b] = (float)(1.0 / bp);
  for (int u = b + 1; u < e; ++u) {
    const double ak = a.coef64[u];
    const double bk = (u == e - 1) ? -a.coef64[u] : (-a.coef64[u] - a.coef64[u + 1]);
    const double bnew = bk - ak * ak / bp;
    a.tw32[u] = (float)(ak / bp);
    bp = bnew;
    a.tib32[u] = (float)(1.0 / bp);
  }
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
template <int QP>
__global__ void __launch_bounds__(kBlock) batch_kernel(BatchArgs a, int do_setup) {
  __shared__ int s_start[kTileCap + 1];
  __shared__ int s_ctop[kTileCap];
  __shared__ int s_nk[kTileCap];
  __shared__ double s_red[4 * (kBlock / 32)];
  const int G = gridDim.x, tid = threadIdx.x, F = a.F;
  SolveCtl* ctl = a.ctl;

  // ======================= setup of new instances =======================
  if (do_setup) {
    // S1: FP32 copies, conditioner, unscaled coefficients, zero vectors
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int i = a.tile_inst[t];
      if (inst_state(a, i) != INST_SETUP) continue;
      TileInfo ti;
      load_tile(a, t, ti, s_start, s_ctop, s_nk);
      const int ncols = ti.c1 - ti.c0;
      const int len = ti.end - ti.base;
      for (int s = tid; s < len; s += kBlock) {
        const int cl = find_col_b(s_start, ncols, s);
        const int j = ti.c0 + cl;
        const int k = s - s_start[cl];
        const int u = ti.base + s;
        const int ctop = s_ctop[cl], nk = s_nk[cl];
        const bool act = k >= ctop;
        const double dz = a.dzz64[u];
        const double Ac = a.colAc[j];
        a.dzz32[u] = (float)dz;
        a.r32[u] = 0.f;
        a.pa32[u] = 0.f;
        a.pb32[u] = 0.f;
        a.x32[u] = 0.f;
        a.z32[u] = 0.f;
        if (QP == 2) a.s32[u] = 0.f;
        if (QP == 1) {
          double c = 1.0;
          if (act) {
            double diag = 0.0;
            for (int f = 0; f < F; ++f) {
              const BFace fc = a.face[(size_t)j * F + f];
              if (fc.ns < 0 || k < fc.kmin || k >= fc.kmax) continue;
              diag += dz * fc.D64;
            }
            const double ak = (k == ctop) ? Ac / dz : 2 * Ac / (dz + a.dzz64[u - 1]);
            if (ctop < nk - 1) {
              if (k == ctop) diag += 2 * ak + 2 * Ac / (a.dzz64[u + 1] + dz);
              else if (k == nk - 1) diag += ak;
              else diag += ak + 2 * Ac / (a.dzz64[u + 1] + dz);
            }
            if (diag <= 0) diag = 1;
            c = sqrt(diag);
          }
          a.c64[u] = c;
          a.cinv32[u] = (float)(1.0 / c);
          a.x64[u] = act ? a.q64[u] * c : 0.0;
          a.b64[u] = act ? a.src64[u] / c : 0.0;
        } else {
          double cf = 0.0;
          if (k == ctop) cf = Ac / dz;
          else if (k > ctop) cf = 2 * Ac / (dz + a.dzz64[u - 1]);
          a.coef64[u] = cf;
          a.coef32[u] = (float)cf;
          a.x64[u] = act ? a.q64[u] : 0.0;
          a.b64[u] = act ? a.src64[u] : 0.0;
        }
      }
      if (QP == 2) {
        __syncthreads();
        for (int c = tid; c < ncols; c += kBlock) column_factor64(a, ti.base + s_start[c], s_ctop[c], s_nk[c]);
      }
      __syncthreads();
    }
    // boundary (non-computational) slots of new instances: fixed values
    for (int i = 0; i < a.ninst; ++i) {
      const BInst& I = a.inst[i];
      if (ld_volatile_int(&I.state) != INST_SETUP) continue;
      for (int u = I.s1 + blockIdx.x * kBlock + tid; u < I.s2; u += G * kBlock) {
        a.x64[u] = a.q64[u];
        a.b64[u] = 0.0;
        a.r32[u] = 0.f;
        a.pa32[u] = 0.f;
        a.pb32[u] = 0.f;
        if (QP == 2) a.s32[u] = 0.f;
        if (QP == 1) {
          a.c64[u] = a.cin64[u];
          a.cinv32[u] = (float)(1.0 / a.cin64[u]);
        }
      }
    }
    if (!grid_sync(ctl, 11, [] {})) return;

    // S2 (qprecond 1): FP64 scaled coefficients (QCoefficients 3427-3452)
    if (QP == 1) {
      for (int t = blockIdx.x; t < a.ntiles; t += G) {
        const int i = a.tile_inst[t];
        if (inst_state(a, i) != INST_SETUP) continue;
        TileInfo ti;
        load_tile(a, t, ti, s_start, s_ctop, s_nk);
        const int ncols = ti.c1 - ti.c0;
        const int len = ti.end - ti.base;
        for (int s = tid; s < len; s += kBlock) {
          const int cl = find_col_b(s_start, ncols, s);
          const int j = ti.c0 + cl;
          const int k = s - s_start[cl];
          const int u = ti.base + s;
          const int ctop = s_ctop[cl];
          const double Ac = a.colAc[j];
          const double dz = a.dzz64[u];
          const double cu = a.c64[u];
          double cf = 0.0;
          if (k == ctop) cf = Ac / dz / cu;
          else if (k > ctop) cf = 2 * Ac / (dz + a.dzz64[u - 1]) / (cu * a.c64[u - 1]);
          a.coef64[u] = cf;
          for (int f = 0; f < F; ++f) {
            const BFace fc = a.face[(size_t)j * F + f];
            double v = 0.0;
            if (fc.ns >= 0 && k >= ctop && k >= fc.kmin && k < fc.kmax) v = dz * fc.D64 / (cu * a.c64[fc.ns + k]);
            a.fc64[(size_t)F * u + f] = v;
          }
        }
        __syncthreads();
      }
      if (!grid_sync(ctl, 12, [] {})) return;
    }

    // S3: initial FP64 residual, first preconditioned residual, alpha0, eps0
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int i = a.tile_inst[t];
      if (inst_state(a, i) != INST_SETUP) continue;
      TileInfo ti;
      load_tile(a, t, ti, s_start, s_ctop, s_nk);
      const int ncols = ti.c1 - ti.c0;
      const int len = ti.end - ti.base;
      double part[2] = {0.0, 0.0};
      for (int s = tid; s < len; s += kBlock) {
        const int cl = find_col_b(s_start, ncols, s);
        const int j = ti.c0 + cl;
        const int k = s - s_start[cl];
        const int u = ti.base + s;
        const int ctop = s_ctop[cl], nk = s_nk[cl];
        if (k < ctop) continue;
        const double r = a.b64[u] - apply64<QP>(a, u, j, k, ctop, nk, a.x64);
        const float rf = (float)r;
        a.r32[u] = rf;
        if (QP == 2) part[1] += r * r;
        else part[0] += f2d(rf) * f2d(rf);
      }
      if (QP == 2) {
        __syncthreads();
        for (int c = tid; c < ncols; c += kBlock) column_solve32(a, ti.base + s_start[c], s_ctop[c], s_nk[c]);
        __syncthreads();
        for (int u = ti.base + tid; u < ti.end; u += kBlock) part[0] += f2d(a.r32[u]) * f2d(a.s32[u]);
      }
      block_sum<2>(part, s_red);
      tile_done<2>(a, t, i, part, s_red, [&](BInst* I, const double* tot) {
        double alpha = tot[0], alpha0 = tot[0];
        if (!I->resnorm) alpha0 = 1;
        const double eps0 = (QP == 2) ? tot[1] : alpha0;
        I->alpha = alpha;
        I->eps0 = eps0;
        I->eps = eps0;
        I->eps_ref = eps0;
        I->mu = 0.0;
        I->nu = 0.0;
        I->n = 0;
        I->nrel = 0;
        I->flags = 0;
        I->par = 0;
        I->status = SGPU_OK;
        I->state = (I->maxiters <= 0 || eps0 == 0) ? INST_DONE : INST_RUN;
      });
    }
    if (!grid_sync(ctl, 13, [&] {
          if (tid == 0) {
            int any = 0;
            for (int i = 0; i < a.ninst; ++i) any |= (a.inst[i].state == INST_RUN);
            a.gflags[3] = any;
            __threadfence();
          }
        }))
      return;
  }

  // ============================ iterations ==============================
  for (int it = 0; it < a.max_iters_chunk; ++it) {
    if (!ld_volatile_int(&a.gflags[3])) break;

    // ---- A: p_new = s + mu p_old (on the fly), z = A p_new, p.z ----
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int i = a.tile_inst[t];
      if (inst_state(a, i) != INST_RUN) continue;
      TileInfo ti;
      load_tile(a, t, ti, s_start, s_ctop, s_nk);
      const BInst& I = a.inst[i];
      const float mu = (float)(*(volatile double*)&I.mu);
      const int par = ld_volatile_int(&I.par);
      const float* pold = par ? a.pb32 : a.pa32;
      float* pnew = par ? a.pa32 : a.pb32;
      const float* S = (QP == 2) ? a.s32 : a.r32;
      const int ncols = ti.c1 - ti.c0;
      const int len = ti.end - ti.base;
      double part[1] = {0.0};
      for (int s = tid; s < len; s += kBlock) {
        const int cl = find_col_b(s_start, ncols, s);
        const int j = ti.c0 + cl;
        const int k = s - s_start[cl];
        const int u = ti.base + s;
        const int ctop = s_ctop[cl], nk = s_nk[cl];
        if (k < ctop) continue;
        const float pu = __fmaf_rn(mu, pold[u], S[u]);
        float y;
        if (QP == 1) {
          const float dz = a.dzz32[u], cu = a.cinv32[u];
          const float Ac = (float)a.colAc[j];
          y = -pu;
          for (int f = 0; f < F; ++f) {
            const BFace fc = a.face[(size_t)j * F + f];
            if (fc.ns < 0 || k < fc.kmin || k >= fc.kmax) continue;
            const int n = fc.ns + k;
            const float pn = __fmaf_rn(mu, pold[n], S[n]);
            y = __fmaf_rn(dz * fc.D * cu * a.cinv32[n], pn, y);
          }
          if (k > ctop) {
            const float pm = __fmaf_rn(mu, pold[u - 1], S[u - 1]);
            const float cf = (2.f * Ac / (dz + a.dzz32[u - 1])) * (cu * a.cinv32[u - 1]);
            y = __fmaf_rn(cf, pm, y);
          }
          if (k < nk - 1) {
            const float pp = __fmaf_rn(mu, pold[u + 1], S[u + 1]);
            const float cf = (2.f * Ac / (a.dzz32[u + 1] + dz)) * (a.cinv32[u + 1] * cu);
            y = __fmaf_rn(cf, pp, y);
          }
        } else {
          y = 0.f;
          for (int f = 0; f < F; ++f) {
            const BFace fc = a.face[(size_t)j * F + f];
            if (fc.ns < 0 || k < fc.kmin || k >= fc.kmax) continue;
            const int n = fc.ns + k;
            const float pn = __fmaf_rn(mu, pold[n], S[n]);
            y = __fmaf_rn(pn - pu, a.dzfD32[fc.es + k], y);
          }
          if (ctop < nk - 1) {
            const float c0 = a.coef32[u];
            if (k == ctop) {
              const float c1 = a.coef32[u + 1];
              const float pp = __fmaf_rn(mu, pold[u + 1], S[u + 1]);
              y += (-2.f * c0 - c1) * pu + c1 * pp;
            } else if (k == nk - 1) {
              const float pm = __fmaf_rn(mu, pold[u - 1], S[u - 1]);
              y += c0 * pm - c0 * pu;
            } else {
              const float c1 = a.coef32[u + 1];
              const float pm = __fmaf_rn(mu, pold[u - 1], S[u - 1]);
              const float pp = __fmaf_rn(mu, pold[u + 1], S[u + 1]);
              y += c0 * pm - (c0 + c1) * pu + c1 * pp;
            }
          } else {
            y -= 2.f * a.coef32[u] * pu;
          }
        }
        a.z32[u] = y;
        pnew[u] = pu;
        part[0] += f2d(pu) * f2d(y);
      }
      block_sum<1>(part, s_red);
      tile_done<1>(a, t, i, part, s_red, [&](BInst* In, const double* tot) {
        const double alpha = In->alpha;
        In->alpha_prev = alpha;
        In->mu = 1 / alpha;  // mu = 1/alpha before nu (2484-2485)
        const double nu = alpha / tot[0];
        In->nu = nu;
        In->par ^= 1;
        if (!isfinite(nu)) {
          In->status = SGPU_BREAKDOWN;
          In->flags = 2;  // final merge
          In->state = INST_DONE;
          atomicOr(&a.gflags[0], 1);
        }
      });
    }
    if (!grid_sync(ctl, 21, [] {})) return;

    // ---- B: x32 += nu p, r -= nu z, preconditioner, r.s, r.r ----
    for (int t = blockIdx.x; t < a.ntiles; t += G) {
      const int i = a.tile_inst[t];
      if (inst_state(a, i) != INST_RUN) continue;
      TileInfo ti;
      const BInst& I = a.inst[i];
      const float nu = (float)(*(volatile double*)&I.nu);
      const float* p = ld_volatile_int(&I.par) ? a.pb32 : a.pa32;
      double part[2] = {0.0, 0.0};
      if (QP == 2) {
        load_tile(a, t, ti, s_start, s_ctop, s_nk);
      } else {
        ti.base = a.col[a.tile_c0[2 * t]].s;
        const BCol cl = a.col[a.tile_c0[2 * t + 1] - 1];
        ti.end = cl.s + cl.nk;
      }
      for (int u = ti.base + tid; u < ti.end; u += kBlock) {
        a.x32[u] = __fmaf_rn(nu, p[u], a.x32[u]);
        const float r = __fmaf_rn(-nu, a.z32[u], a.r32[u]);
        a.r32[u] = r;
        if (QP != 2) part[0] += f2d(r) * f2d(r);
      }
      if (QP == 2) {
        __syncthreads();
        const int ncols = a.tile_c0[2 * t + 1] - a.tile_c0[2 * t];
        for (int c = tid; c < ncols; c += kBlock) column_solve32(a, ti.base + s_start[c], s_ctop[c], s_nk[c]);
        __syncthreads();
        for (int u = ti.base + tid; u < ti.end; u += kBlock) {
          const float r = a.r32[u];
          part[0] += f2d(r) * f2d(a.s32[u]);
          part[1] += f2d(r) * f2d(r);
        }
      }
      block_sum<2>(part, s_red);
      tile_done<2>(a, t, i, part, s_red, [&](BInst* In, const double* tot) {
        const double alpha = tot[0];
        const double mu = In->mu * alpha;  // mu *= alpha (2498/2509)
        In->mu = mu;
        In->alpha = alpha;
        const double eps = (QP == 2) ? tot[1] : alpha;
        In->eps = eps;
        const int n = In->n + 1;
        In->n = n;
        int flags = 0;
        if (!isfinite(alpha) || !isfinite(mu)) {
          In->status = SGPU_BREAKDOWN;
          In->state = INST_DONE;
          flags = 2;
        } else if (eps == 0) {
          In->state = INST_DONE;
          flags = 2;
        } else if (eps < In->tol2 * In->eps0 || eps < a.delta2 * In->eps_ref) {
          flags = 1;  // verify / refresh with the FP64 true residual
        } else if (n >= In->maxiters) {
          In->status = SGPU_MAXITER;
          In->state = INST_DONE;
          flags = 2;
        }
        if (flags == 1 && n >= In->maxiters) flags = 1 | 4;  // last chance: verify, else stop
        In->flags = flags;
        if (flags) atomicOr(&a.gflags[0], 1);
      });
    }
    if (!grid_sync(ctl, 22, [&] {
          if (tid == 0) {
            a.gflags[2] = a.gflags[0];
            a.gflags[0] = 0;
            __threadfence();
          }
        }))
      return;

    if (ld_volatile_int(&a.gflags[2])) {
      // ---- R1: x64 += x32, x32 = 0 for flagged instances ----
      for (int t = blockIdx.x; t < a.ntiles; t += G) {
        const int i = a.tile_inst[t];
        if (!inst_flags(a, i)) continue;
        const int base = a.col[a.tile_c0[2 * t]].s;
        const BCol cl = a.col[a.tile_c0[2 * t + 1] - 1];
        const int end = cl.s + cl.nk;
        for (int u = base + tid; u < end; u += kBlock) {
          a.x64[u] += f2d(a.x32[u]);
          a.x32[u] = 0.f;
        }
      }
      if (!grid_sync(ctl, 23, [] {})) return;
      // ---- R2: FP64 true residual for instances that verify / refresh ----
      for (int t = blockIdx.x; t < a.ntiles; t += G) {
        const int i = a.tile_inst[t];
        const int fl = inst_flags(a, i);
        if (!fl) continue;
        if (!(fl & 1)) {
          // final merge only: finish the tile count so the flags get cleared
          double part[2] = {0.0, 0.0};
          tile_done<2>(a, t, i, part, s_red, [&](BInst* In, const double*) { In->flags = 0; });
          continue;
        }
        TileInfo ti;
        load_tile(a, t, ti, s_start, s_ctop, s_nk);
        const int ncols = ti.c1 - ti.c0;
        const int len = ti.end - ti.base;
        double part[2] = {0.0, 0.0};
        for (int s = tid; s < len; s += kBlock) {
          const int cl = find_col_b(s_start, ncols, s);
          const int j = ti.c0 + cl;
          const int k = s - s_start[cl];
          const int u = ti.base + s;
          const int ctop = s_ctop[cl], nk = s_nk[cl];
          if (k < ctop) continue;
          const double r = a.b64[u] - apply64<QP>(a, u, j, k, ctop, nk, a.x64);
          const float rf = (float)r;
          a.r32[u] = rf;
          if (QP == 2) part[1] += r * r;
          else part[0] += r * r;
        }
        if (QP == 2) {
          __syncthreads();
          for (int c = tid; c < ncols; c += kBlock) column_solve32(a, ti.base + s_start[c], s_ctop[c], s_nk[c]);
          __syncthreads();
          for (int u = ti.base + tid; u < ti.end; u += kBlock) part[0] += f2d(a.r32[u]) * f2d(a.s32[u]);
        }
        block_sum<2>(part, s_red);
        tile_done<2>(a, t, i, part, s_red, [&](BInst* In, const double* tot) {
          const double alpha = tot[0];
          const double eps = (QP == 2) ? tot[1] : alpha;
          In->nrel += 1;
          In->eps = eps;
          In->eps_ref = eps;
          if (eps < In->tol2 * In->eps0 || eps == 0) {
            In->state = INST_DONE;
          } else if (In->flags & 4) {
            In->status = SGPU_MAXITER;
            In->state = INST_DONE;
          } else {
            In->mu = alpha / In->alpha_prev;  // beta from the true residual
            In->alpha = alpha;
          }
          In->flags = 0;
        });
      }
      if (!grid_sync(ctl, 24, [&] {
            if (tid == 0) {
              int any = 0;
              for (int i = 0; i < a.ninst; ++i) any |= (a.inst[i].state == INST_RUN);
              a.gflags[3] = any;
              __threadfence();
            }
          }))
        return;
    }
  }
}

// ---------------------------------------------------------------------------
// host side: the batch engine
// ---------------------------------------------------------------------------
struct Range {
  long long off = 0, len = 0;
};

// first-fit allocator over [0, cap)
struct Arena {
  long long cap = 0;
  std::vector<Range> freel;
  void init(long long c) {
    cap = c;
    freel.assign(1, Range{0, c});
  }
  long long alloc(long long n) {
    if (n <= 0) return 0;
    for (size_t i = 0; i < freel.size(); ++i)
      if (freel[i].len >= n) {
        long long o = freel[i].off;
        freel[i].off += n;
        freel[i].len -= n;
        if (freel[i].len == 0) freel.erase(freel.begin() + i);
        return o;
      }
    return -1;
  }
  void release(long long off, long long n) {
    if (n <= 0) return;
    freel.push_back(Range{off, n});
    std::sort(freel.begin(), freel.end(), [](const Range& x, const Range& y) { return x.off < y.off; });
    std::vector<Range> m;
    for (auto& r : freel) {
      if (!m.empty() && m.back().off + m.back().len == r.off) m.back().len += r.len;
      else m.push_back(r);
    }
    freel.swap(m);
  }
  long long free_total() const {
    long long s = 0;
    for (auto& r : freel) s += r.len;
    return s;
  }
};

struct HostInst {
  bool live = false;
  int id = -1;
  long long s_off = 0, n3 = 0, n3c = 0;  // slots
  long long c_off = 0, ncomp = 0;        // columns
  long long e_off = 0, ne3 = 0;          // edge slots
  int Nc = 0;
  std::vector<int> dev2cell, Nk, ctop, coff;  // device column -> cell, per cell Nk/ctop, device column offsets
  std::vector<int> tiles_rel;                  // tile boundaries (relative column index), size ntiles+1
  int qprecond = 1;
  double tol = 1e-10;
  int maxiters = 1000;
  double resnorm = 1.0;
  bool done_reported = false;
};

}  // namespace sgpu

using namespace sgpu;

struct sgpu_batch {
  int device = 0;
  int qprecond = 1;
  int F = 3;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  long long timeout_ns = 2000000000LL;
  int grid_override = 0;
  double delta = 0.01;
  long long max_slots = 0, max_cols = 0, max_eslots = 0;
  int max_inst = 0, max_tiles = 0;
  Arena slots, cols, eslots;
  std::vector<HostInst> inst;
  std::vector<BInst> h_inst;
  bool pending_setup = false;
  // device
  std::vector<void*> allocs;
  BatchArgs a{};
  int* d_tile_c0 = nullptr;
  int* d_tile_inst = nullptr;
  BCol* d_col = nullptr;
  BFace* d_face = nullptr;
  double* d_colAc = nullptr;
  double *d_dzz64 = nullptr, *d_src64 = nullptr, *d_q64 = nullptr, *d_cin64 = nullptr, *d_dzfD64 = nullptr;
  BInst* d_inst = nullptr;
  SolveCtl* d_ctl = nullptr;
  int* d_gflags = nullptr;
  SolveCtl* h_ctl = nullptr;
  int ntiles = 0;
  std::vector<int> h_tile_c0, h_tile_inst;
  double last_ms = 0.0;
  long long last_work = 0;
};

static int bfail(sgpu_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(call)                                                                                          \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? SGPU_OOM : SGPU_CUDA_ERROR, "%s: %s (line %d)", #call, \
                   cudaGetErrorString(e_), __LINE__);                                                      \
  } while (0)

template <class T>
static int balloc(sgpu_batch* b, T** p, size_t n) {
  void* v = nullptr;
  BCK(cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T)));
  b->allocs.push_back(v);
  *p = (T*)v;
  return SGPU_OK;
}

namespace {
struct Guard {
  int prev = -1;
  explicit Guard(int d) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(d);
  }
  ~Guard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};
}  // namespace

static int batch_max_grid(int qp, int dev) {
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* fn = qp == 1 ? (const void*)batch_kernel<1> : qp == 2 ? (const void*)batch_kernel<2>
                                                                      : (const void*)batch_kernel<0>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kBlock, 0) != cudaSuccess) return 0;
  return sms * per;
}

extern "C" {

int sgpu_batch_create(int device, int qprecond, int maxfaces, long long max_slots, long long max_cols,
                      long long max_edge_slots, int max_instances, sgpu_batch** out) {
  if (!out || qprecond < 0 || qprecond > 2 || maxfaces < 1 || maxfaces > kMaxF || max_slots <= 0 ||
      max_cols <= 0 || max_instances <= 0 || max_slots > 0x7ffffff0LL || max_edge_slots > 0x7ffffff0LL)
    return SGPU_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return SGPU_NO_DEVICE;
  if (device < 0 || device >= ndev) return SGPU_BAD_ARG;
  sgpu_batch* b = new sgpu_batch();
  *out = b;
  b->device = device;
  b->qprecond = qprecond;
  b->F = maxfaces;
  b->max_slots = max_slots;
  b->max_cols = max_cols;
  b->max_eslots = std::max(1LL, max_edge_slots);
  b->max_inst = max_instances;
  b->max_tiles = (int)std::min<long long>(0x7fffffff, max_cols + max_slots / kTileCap + 2);
  b->slots.init(max_slots);
  b->cols.init(max_cols);
  b->eslots.init(b->max_eslots);
  b->inst.resize(max_instances);
  b->h_inst.assign(max_instances, BInst{});
  Guard g(device);
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaEventCreate(&b->ev0));
  BCK(cudaEventCreate(&b->ev1));
  BCK(cudaMallocHost((void**)&b->h_ctl, sizeof(SolveCtl)));
  const size_t S = (size_t)max_slots + 1, E = (size_t)b->max_eslots + 1, Cn = (size_t)max_cols + 1;
  int rc;
  BatchArgs& a = b->a;
  a.F = maxfaces;
  if ((rc = balloc(b, &b->d_tile_c0, 2 * ((size_t)b->max_tiles + 1)))) return rc;
  if ((rc = balloc(b, &b->d_tile_inst, (size_t)b->max_tiles + 1))) return rc;
  if ((rc = balloc(b, &b->d_col, Cn))) return rc;
  if ((rc = balloc(b, &b->d_face, Cn * maxfaces))) return rc;
  if ((rc = balloc(b, &b->d_colAc, Cn))) return rc;
  if ((rc = balloc(b, &b->d_dzz64, S))) return rc;
  if ((rc = balloc(b, &b->d_src64, S))) return rc;
  if ((rc = balloc(b, &b->d_q64, S))) return rc;
  if ((rc = balloc(b, &b->d_cin64, S))) return rc;
  if ((rc = balloc(b, &b->d_dzfD64, E))) return rc;
  if ((rc = balloc(b, &a.c64, S))) return rc;
  if ((rc = balloc(b, &a.coef64, S))) return rc;
  if (qprecond == 1 && (rc = balloc(b, &a.fc64, S * maxfaces))) return rc;
  if ((rc = balloc(b, &a.x64, S))) return rc;
  if ((rc = balloc(b, &a.b64, S))) return rc;
  if ((rc = balloc(b, &a.dzz32, S))) return rc;
  if ((rc = balloc(b, &a.cinv32, S))) return rc;
  if ((rc = balloc(b, &a.coef32, S))) return rc;
  if ((rc = balloc(b, &a.dzfD32, E))) return rc;
  if (qprecond == 2) {
    if ((rc = balloc(b, &a.tw32, S))) return rc;
    if ((rc = balloc(b, &a.tib32, S))) return rc;
    if ((rc = balloc(b, &a.s32, S))) return rc;
  }
  if ((rc = balloc(b, &a.r32, S))) return rc;
  if ((rc = balloc(b, &a.pa32, S))) return rc;
  if ((rc = balloc(b, &a.pb32, S))) return rc;
  if ((rc = balloc(b, &a.x32, S))) return rc;
  if ((rc = balloc(b, &a.z32, S))) return rc;
  if ((rc = balloc(b, &a.tpart, 2 * ((size_t)b->max_tiles + 1)))) return rc;
  if ((rc = balloc(b, &b->d_inst, (size_t)max_instances))) return rc;
  if ((rc = balloc(b, &b->d_ctl, 1))) return rc;
  if ((rc = balloc(b, &b->d_gflags, 4))) return rc;
  BCK(cudaMemsetAsync(a.coef64, 0, S * sizeof(double), b->stream));
  BCK(cudaMemsetAsync(b->d_cin64, 0, S * sizeof(double), b->stream));
  BCK(cudaMemsetAsync(b->d_inst, 0, sizeof(BInst) * max_instances, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  a.tile_c0 = b->d_tile_c0;
  a.tile_inst = b->d_tile_inst;
  a.col = b->d_col;
  a.face = b->d_face;
  a.colAc = b->d_colAc;
  a.dzz64 = b->d_dzz64;
  a.src64 = b->d_src64;
  a.q64 = b->d_q64;
  a.cin64 = b->d_cin64;
  a.dzfD64 = b->d_dzfD64;
  a.inst = b->d_inst;
  a.ctl = b->d_ctl;
  a.gflags = b->d_gflags;
  return SGPU_OK;
}

int sgpu_batch_destroy(sgpu_batch* b) {
  if (!b) return SGPU_BAD_ARG;
  {
    Guard g(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (void* p : b->allocs) cudaFree(p);
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
  }
  delete b;
  return SGPU_OK;
}

const char* sgpu_batch_last_error(const sgpu_batch* b) { return b ? b->err.c_str() : "null batch"; }

long long sgpu_batch_bytes_per_request(int qprecond, int maxfaces, long long n3, long long ncols,
                                       long long nedge_slots) {
  // device bytes an instance occupies (layout of sgpu_batch_create's arrays)
  long long per_slot = 8 * 7 + 4 * 8 + (qprecond == 1 ? 8LL * maxfaces : 0) + (qprecond == 2 ? 12 : 0);
  long long per_col = (long long)sizeof(BCol) + (long long)sizeof(BFace) * maxfaces + 8;
  long long per_eslot = 12;
  return per_slot * n3 + per_col * ncols + per_eslot * nedge_slots + 16 * (ncols + n3 / kTileCap + 2);
}

int sgpu_batch_add(sgpu_batch* b, const sgpu_grid_desc* g, const int* ctop, const double* const* dzz,
                   const double* const* dzf, const double* D, const double* const* q, const double* const* src,
                   const double* const* c, double qepsilon, int qmaxiters, double resnorm, int* id_out) {
  if (!b || !g || !ctop || !dzz || !dzf || !D || !q || !src || !id_out) return SGPU_BAD_ARG;
  if (g->maxfaces != b->F) return bfail(b, SGPU_BAD_ARG, "maxfaces %d differs from the batch's %d", g->maxfaces, b->F);
  const int Nc = g->Nc, Ne = g->Ne, F = g->maxfaces;
  const int* cd = g->celldist;
  if (Nc <= 0 || !cd || !(cd[0] == 0 && cd[0] <= cd[1] && cd[1] <= cd[2] && cd[2] <= Nc) || cd[1] == 0)
    return bfail(b, SGPU_BAD_GRID, "celldist must satisfy 0 = c0 < c1 <= c2 <= Nc");
  if (g->Nkmax > kTileCap) return bfail(b, SGPU_BAD_GRID, "Nkmax %d exceeds %d", g->Nkmax, kTileCap);
  int id = -1;
  for (int i = 0; i < b->max_inst; ++i)
    if (!b->inst[i].live) {
      id = i;
      break;
    }
  if (id < 0) return bfail(b, SGPU_OOM, "no free instance slot (max %d)", b->max_inst);
  HostInst H;
  H.live = true;
  H.id = id;
  H.Nc = Nc;
  H.Nk.assign(g->Nk, g->Nk + Nc);
  H.ctop.assign(ctop, ctop + Nc);
  // device order: cellp[0..c2) then the rest
  std::vector<int> c2d(Nc, -1);
  for (int t = 0; t < cd[2]; ++t) {
    const int i = g->cellp[t];
    if (i < 0 || i >= Nc || c2d[i] >= 0) return bfail(b, SGPU_BAD_GRID, "cellp invalid or repeated");
    c2d[i] = (int)H.dev2cell.size();
    H.dev2cell.push_back(i);
  }
  for (int i = 0; i < Nc; ++i)
    if (c2d[i] < 0) {
      c2d[i] = (int)H.dev2cell.size();
      H.dev2cell.push_back(i);
    }
  H.coff.assign(Nc + 1, 0);
  long long acc = 0;
  for (int j = 0; j < Nc; ++j) {
    const int i = H.dev2cell[j];
    if (g->Nk[i] < 1 || g->Nk[i] > g->Nkmax || ctop[i] < 0 || ctop[i] >= g->Nk[i])
      return bfail(b, SGPU_BAD_GRID, "Nk/ctop out of range at cell %d", i);
    H.coff[j] = (int)acc;
    acc += g->Nk[i];
  }
  H.coff[Nc] = (int)acc;
  H.n3 = acc;
  H.ncomp = cd[1];
  H.n3c = H.coff[cd[1]];
  std::vector<long long> eoff(Ne + 1, 0);
  for (int e = 0; e < Ne; ++e) eoff[e + 1] = eoff[e] + g->Nke[e];
  H.ne3 = eoff[Ne];
  H.qprecond = b->qprecond;
  H.tol = qepsilon;
  H.maxiters = qmaxiters;
  H.resnorm = resnorm;
  // tiles over the computational columns (relative)
  H.tiles_rel.push_back(0);
  int cur = 0;
  for (int j = 0; j < cd[1]; ++j) {
    const int len = g->Nk[H.dev2cell[j]];
    if (cur + len > kTileCap) {
      H.tiles_rel.push_back(j);
      cur = 0;
    }
    cur += len;
  }
  H.tiles_rel.push_back(cd[1]);
  // reserve device ranges
  H.s_off = b->slots.alloc(H.n3);
  H.c_off = b->cols.alloc(H.ncomp);
  H.e_off = b->eslots.alloc(std::max(1LL, H.ne3));
  if (H.s_off < 0 || H.c_off < 0 || H.e_off < 0) {
    if (H.s_off >= 0) b->slots.release(H.s_off, H.n3);
    if (H.c_off >= 0) b->cols.release(H.c_off, H.ncomp);
    if (H.e_off >= 0) b->eslots.release(H.e_off, std::max(1LL, H.ne3));
    return bfail(b, SGPU_OOM, "batch capacity exhausted (slots %lld free of %lld)", b->slots.free_total(),
                 b->max_slots);
  }
  // stage host data (pageable copies; the upload is synchronous per instance)
  Guard gd(b->device);
  std::vector<double> v_dzz(H.n3), v_src(H.n3), v_q(H.n3), v_c(H.n3, 1.0), v_dzfD(std::max(1LL, H.ne3));
  for (int j = 0; j < Nc; ++j) {
    const int i = H.dev2cell[j];
    std::memcpy(&v_dzz[H.coff[j]], dzz[i], sizeof(double) * g->Nk[i]);
    std::memcpy(&v_src[H.coff[j]], src[i], sizeof(double) * g->Nk[i]);
    std::memcpy(&v_q[H.coff[j]], q[i], sizeof(double) * g->Nk[i]);
    if (c) std::memcpy(&v_c[H.coff[j]], c[i], sizeof(double) * g->Nk[i]);
  }
  for (int e = 0; e < Ne; ++e)
    for (int k = 0; k < g->Nke[e]; ++k) v_dzfD[eoff[e] + k] = dzf[e][k] * D[e];
  std::vector<BCol> v_col(H.ncomp);
  std::vector<BFace> v_face((size_t)H.ncomp * F);
  std::vector<double> v_Ac(H.ncomp);
  for (int j = 0; j < cd[1]; ++j) {
    const int i = H.dev2cell[j];
    v_col[j].s = (int)(H.s_off + H.coff[j]);
    v_col[j].nk = g->Nk[i];
    v_col[j].ctop = ctop[i];
    v_col[j].inst = id;
    v_Ac[j] = g->Ac[i];
    for (int f = 0; f < F; ++f) {
      BFace& fc = v_face[(size_t)j * F + f];
      fc.ns = -1;
      fc.es = 0;
      fc.kmin = fc.kmax = 0;
      fc.D = 0.f;
      fc.D64 = 0.0;
      if (f >= g->nfaces[i]) continue;
      const int nc = g->neigh[i * F + f], e = g->face[i * F + f];
      if (nc < 0) continue;
      if (e < 0 || e >= Ne || nc >= Nc) return bfail(b, SGPU_BAD_GRID, "face/neigh out of range at cell %d", i);
      if (g->Nke[e] > g->Nk[i] || g->Nke[e] > g->Nk[nc]) return bfail(b, SGPU_BAD_GRID, "Nke exceeds Nk at edge %d", e);
      fc.ns = (int)(H.s_off + H.coff[c2d[nc]]);
      fc.es = (int)(H.e_off + eoff[e]);
      fc.kmin = (short)std::max(ctop[i], ctop[nc]);
      fc.kmax = (short)g->Nke[e];
      fc.D = (float)D[e];
      fc.D64 = D[e];
    }
  }
  std::vector<float> v_dzfD32(v_dzfD.size());
  for (size_t k = 0; k < v_dzfD.size(); ++k) v_dzfD32[k] = (float)v_dzfD[k];
  cudaStream_t s = b->stream;
  BCK(cudaMemcpyAsync(b->d_dzz64 + H.s_off, v_dzz.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_src64 + H.s_off, v_src.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_q64 + H.s_off, v_q.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_cin64 + H.s_off, v_c.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  if (H.ne3 > 0) {
    BCK(cudaMemcpyAsync(b->d_dzfD64 + H.e_off, v_dzfD.data(), 8 * H.ne3, cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->a.dzfD32 + H.e_off, v_dzfD32.data(), 4 * H.ne3, cudaMemcpyHostToDevice, s));
  }
  BCK(cudaMemcpyAsync(b->d_col + H.c_off, v_col.data(), sizeof(BCol) * H.ncomp, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_face + H.c_off * F, v_face.data(), sizeof(BFace) * H.ncomp * F, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_colAc + H.c_off, v_Ac.data(), 8 * H.ncomp, cudaMemcpyHostToDevice, s));
  BCK(cudaStreamSynchronize(s));
  BInst& I = b->h_inst[id];
  std::memset(&I, 0, sizeof(BInst));
  I.s0 = (int)(H.s_off);
  I.s1 = (int)(H.s_off + H.n3c);
  I.s2 = (int)(H.s_off + H.n3);
  I.maxiters = qmaxiters;
  I.qprecond = b->qprecond;
  I.tol2 = qepsilon * qepsilon;
  I.resnorm = resnorm;
  I.state = INST_SETUP;
  I.status = SGPU_OK;
  b->inst[id] = std::move(H);
  b->pending_setup = true;
  *id_out = id;
  return SGPU_OK;
}

// Runs up to max_iters global iterations (<= 0: until every instance is done).
// Returns the number of instances still running in *running.
int sgpu_batch_run(sgpu_batch* b, int max_iters, int* running, double* ms, long long* unknown_iters) {
  if (!b) return SGPU_BAD_ARG;
  Guard gd(b->device);
  // tile table of live, unfinished instances
  b->h_tile_c0.clear();
  b->h_tile_inst.clear();
  int ninst = 0;
  std::vector<int> n_before(b->max_inst, 0);
  for (int i = 0; i < b->max_inst; ++i) {
    HostInst& H = b->inst[i];
    BInst& I = b->h_inst[i];
    if (!H.live) continue;
    ninst = i + 1;
    if (I.state != INST_SETUP && I.state != INST_RUN) {
      I.t0 = I.t1 = 0;
      continue;
    }
    n_before[i] = I.state == INST_RUN ? I.n : 0;
    I.t0 = (int)b->h_tile_c0.size();
    for (size_t k = 0; k + 1 < H.tiles_rel.size(); ++k) {
      b->h_tile_c0.push_back((int)(H.c_off + H.tiles_rel[k]));
      b->h_tile_inst.push_back(i);
    }
    I.t1 = (int)b->h_tile_c0.size();
    I.cnt = 0;
  }
  const int ntiles = (int)b->h_tile_c0.size();
  if (ntiles > b->max_tiles) return bfail(b, SGPU_OOM, "too many tiles");
  if (ntiles == 0) {
    if (running) *running = 0;
    if (ms) *ms = 0;
    if (unknown_iters) *unknown_iters = 0;
    return SGPU_OK;
  }
  // tiles as (first column, end column) pairs: an instance's last tile ends at its last column
  std::vector<int> table(2 * ntiles), tinst(ntiles);
  for (int t = 0; t < ntiles; ++t) {
    const int i = b->h_tile_inst[t];
    tinst[t] = i;
    const bool same = t + 1 < ntiles && b->h_tile_inst[t + 1] == i;
    table[2 * t] = b->h_tile_c0[t];
    table[2 * t + 1] = same ? b->h_tile_c0[t + 1] : (int)(b->inst[i].c_off + b->inst[i].ncomp);
  }
  b->ntiles = ntiles;
  BCK(cudaMemcpyAsync(b->d_tile_c0, table.data(), sizeof(int) * 2 * ntiles, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_tile_inst, tinst.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_inst, b->h_inst.data(), sizeof(BInst) * ninst, cudaMemcpyHostToDevice, b->stream));
  std::memset(b->h_ctl, 0, sizeof(SolveCtl));
  b->h_ctl->timeout_ns = b->timeout_ns;
  BCK(cudaMemcpyAsync(b->d_ctl, b->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, b->stream));
  int any_run = 0;
  for (int i = 0; i < ninst; ++i) any_run |= (b->inst[i].live && b->h_inst[i].state == INST_RUN);
  int gfl[4] = {0, 0, 0, any_run};
  BCK(cudaMemcpyAsync(b->d_gflags, gfl, sizeof gfl, cudaMemcpyHostToDevice, b->stream));
  BatchArgs a = b->a;
  a.F = b->F;
  a.ntiles = ntiles;
  a.ninst = ninst;
  a.max_iters_chunk = max_iters > 0 ? max_iters : 0x7fffffff;
  a.delta2 = b->delta * b->delta;
  int maxg = batch_max_grid(b->qprecond, b->device);
  if (maxg <= 0) return bfail(b, SGPU_CUDA_ERROR, "occupancy query failed");
  int grid = b->grid_override > 0 ? std::min(b->grid_override, maxg) : maxg;
  grid = std::max(1, std::min(grid, ntiles));
  int do_setup = b->pending_setup ? 1 : 0;
  void* args[] = {(void*)&a, (void*)&do_setup};
  const void* fn = b->qprecond == 1 ? (const void*)batch_kernel<1>
                 : b->qprecond == 2 ? (const void*)batch_kernel<2> : (const void*)batch_kernel<0>;
  BCK(cudaEventRecord(b->ev0, b->stream));
  BCK(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0, b->stream));
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaMemcpyAsync(b->h_inst.data(), b->d_inst, sizeof(BInst) * ninst, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->pending_setup = false;
  float fms = 0.f;
  cudaEventElapsedTime(&fms, b->ev0, b->ev1);
  b->last_ms = fms;
  if (b->h_ctl->status == SGPU_TIMEOUT)
    return bfail(b, SGPU_TIMEOUT, "device barrier wait timed out in phase %d", b->h_ctl->phase_err);
  int run = 0;
  long long work = 0;
  for (int i = 0; i < ninst; ++i) {
    if (!b->inst[i].live) continue;
    const BInst& I = b->h_inst[i];
    run += I.state == INST_RUN || I.state == INST_SETUP;
    long long unk = 0;
    const HostInst& H = b->inst[i];
    for (int j = 0; j < H.ncomp; ++j) unk += H.Nk[H.dev2cell[j]] - H.ctop[H.dev2cell[j]];
    work += unk * (long long)(I.n - n_before[i]);
  }
  b->last_work = work;
  if (running) *running = run;
  if (ms) *ms = fms;
  if (unknown_iters) *unknown_iters = work;
  return SGPU_OK;
}

// Copies an instance's result to the caller's jagged q (computational cells,
// levels [ctop, Nk)) and its report; frees the instance when `release` != 0.
int sgpu_batch_result(sgpu_batch* b, int id, double* const* q, sgpu_stats* st, int release) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live) return SGPU_BAD_ARG;
  HostInst& H = b->inst[id];
  const BInst& I = b->h_inst[id];
  if (st) {
    st->status = I.status;
    st->niters = I.n;
    st->eps = I.eps;
    st->eps0 = I.eps0;
    st->ms_solve = b->last_ms;
    st->ms_total = 0;
    long long unk = 0;
    for (int j = 0; j < H.ncomp; ++j) unk += H.Nk[H.dev2cell[j]] - H.ctop[H.dev2cell[j]];
    st->unknowns = unk;
  }
  if (q) {
    if (I.state != INST_DONE) return bfail(b, SGPU_BAD_ARG, "instance %d has not finished", id);
    Guard gd(b->device);
    std::vector<double> x(H.n3c), c(H.n3c, 1.0);
    BCK(cudaMemcpyAsync(x.data(), b->a.x64 + H.s_off, 8 * H.n3c, cudaMemcpyDeviceToHost, b->stream));
    if (b->qprecond == 1)
      BCK(cudaMemcpyAsync(c.data(), b->a.c64 + H.s_off, 8 * H.n3c, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    for (int j = 0; j < H.ncomp; ++j) {
      const int i = H.dev2cell[j];
      for (int k = H.ctop[i]; k < H.Nk[i]; ++k) {
        const int u = H.coff[j] + k;
        q[i][k] = b->qprecond == 1 ? x[u] / c[u] : x[u];
      }
    }
  }
  if (release) {
    b->slots.release(H.s_off, H.n3);
    b->cols.release(H.c_off, H.ncomp);
    b->eslots.release(H.e_off, std::max(1LL, H.ne3));
    H = HostInst();
    std::memset(&b->h_inst[id], 0, sizeof(BInst));
  }
  return SGPU_OK;
}

int sgpu_batch_state(const sgpu_batch* b, int id) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live) return -1;
  return b->h_inst[id].state;
}

int sgpu_batch_set(sgpu_batch* b, double delta, int grid, long long timeout_ns) {
  if (!b) return SGPU_BAD_ARG;
  if (delta > 0) b->delta = delta;
  if (grid >= 0) b->grid_override = grid;
  if (timeout_ns > 0) b->timeout_ns = timeout_ns;
  return SGPU_OK;
}

void* sgpu_batch_stream(sgpu_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"
