// sgpu_h.cu -- the free-surface PCG (CGSolve) as one persistent, cooperative
// kernel per solve, FP64 throughout.
//
// Reference semantics followed (main/phys.c of SUNTANS):
//   CGSolve          3086-3217  type-3 boundary lift (3102-3134), Jacobi or
//                               plain CG, stop at sqrt(eps/eps0) < epsilon,
//                               loop guard eps != 0 && alpha != 0
//   HPreconditioner  3227-3235  y = x / hcoef
//   HCoefficients    3252-3269  fcoef = tmp*D*df/dg, coef = Ac + sum fcoef
//   InnerProduct     3280-3294
//   OperatorH        3335-3349  y = coef*x - sum fcoef*x[neigh]
//
// Layout: cells in device order (computational first, then type-3 boundary
// cells, then the rest).  Face f of cell j: coefficient hf[f*ncomp + j] and
// neighbour hn[f*ncomp + j]; a missing face points at the cell itself with a
// zero coefficient, so the apply has no branches.  The whole 2-D problem
// (about 110 bytes per cell) stays in L2 for up to ~1M cells, so the kernel is
// bound by GB300's FP64 rate (about 2 FP64 FMAs per SM and cycle) and by its
// grid barriers, not by HBM.  Three choices follow from that:
//   * two barriers per iteration instead of three: the direction
//     p = s + mu p_old (s = r/hcoef or r) is formed inside the apply, for the
//     cell and for each neighbour it reads, from a double-buffered p_old, so the
//     separate direction sweep and its barrier go;
//   * the Jacobi step multiplies by 1/hcoef, formed once per solve, instead of
//     dividing every iteration (an FP64 division costs ~20 FP64 instructions
//     on GB300); the product differs from the quotient by at most one rounding;
//   * the barrier is a plain arrive-and-wait on a monotonic counter and every
//     CTA reduces the per-CTA partials itself in the same fixed order, so the
//     scalars (nu, mu, alpha, eps) are the same bits in every CTA without a
//     second round trip through one finalising CTA (publishing the partials
//     themselves as the arrival, with every CTA polling all of them, measured
//     slower: the polling contends in L2);
//   * few, large CTAs (kHBlock threads, one per SM): the cost of a barrier
//     grows with the number of CTAs arriving, and each thread works on two
//     cells at a time so that their L2 gathers overlap;
//   * each CTA owns a contiguous range of cells (Morton order keeps most
//     neighbours inside it): it forms the direction of its own cells once,
//     into shared memory, and forms it on the fly only for neighbours owned
//     by another CTA; z stays in shared memory between the two phases;
//   * the scalar recurrences (divisions, the square root of the stopping
//     test) run on one thread per CTA and are broadcast through shared
//     memory -- on every thread they cost several microseconds of FP64 pipe
//     per barrier;
//   * the inner products are reduced with few FP64 instructions (cta_sum,
//     grid_sum): with shuffle trees in every warp and every thread summing
//     the warp results, the reductions took more of the FP64 pipe than the CG
//     arithmetic itself (ncu: DADD 60% of the FP64 instructions).
// The scalar recurrences are CGSolve's: mu = 1/alpha, nu = alpha/(p.z),
// mu *= alpha_new, p = s + mu p.
#include "sgpu_common.cuh"
#include "sgpu_q.h"

namespace sgpu {

#ifndef SGPU_H_BLOCK
#define SGPU_H_BLOCK 512
#endif
constexpr int kHBlock = SGPU_H_BLOCK;  // threads per CTA of the free-surface kernel (one CTA per SM)
constexpr size_t kHStaticSmem = sizeof(double) * (2 * kHBlock + 2 + 8) + 64;
// the CTA's cells' vectors and coefficients: what the 227 KB a CTA may hold
// leaves beside the static arrays
constexpr size_t kHMaxDynSmem = (227 * 1024 - kHStaticSmem) & ~(size_t)1023;

// The per-thread cell loop over [b, e) with step BS, two cells per step so
// that their gathers are in flight together: body(j0, j1, two) with j1 valid
// only when two is true.
template <class Body>
__device__ __forceinline__ void cells2(int b, int e, int step, Body&& body) {
  int j = b;
  for (; j + step < e; j += 2 * step) body(j, j + step, true);
  if (j < e) body(j, j, false);
}

// The direction p = s + mu p_old of cell k, with one rounding (the same bits
// wherever it is formed).
__device__ __forceinline__ double hdir(const double* __restrict__ sv, const double* __restrict__ po, double mu,
                                       int k) {
  return __fma_rn(mu, po[k], sv[k]);
}

// SM: the CTA's directions, z and constant coefficients live in shared memory
// (cells per CTA few enough); otherwise every direction is formed on the fly
// and everything is read from and written to global memory.
template <int HP, bool SM>
__global__ void __launch_bounds__(kHBlock, 1) cgsolve_kernel(HArgs a) {
  // SM: the CTA's directions [0, C), z [C, 2C), hcoef [2C, 3C), 1/hcoef
  // [3C, 4C), face coefficients [4C, (4+F)C) and neighbours (ints) after them
  extern __shared__ double s_dyn[];
  __shared__ double s_red[2 * kHBlock + 2];
  __shared__ double s_sc[8];  // scalars from thread 0: mu, nu, done
  SolveCtl* ctl = a.ctl;
  const int G = gridDim.x;
  const int tid = threadIdx.x;
  const int F = a.F;
  const int nc = a.ncomp;
  const int C = a.cpc;
  const int lo = min(nc, blockIdx.x * C), hi = min(nc, lo + C);
  unsigned int nbar = 0;  // barriers passed
  double* partA = a.partials;          // [2][G]: p.z
  double* partB = a.partials + 2 * G;  // [2][2][G]: r.s, r.r
  double* sp = s_dyn;
  double* sz = s_dyn + C;
  double* shc = s_dyn + 2 * (size_t)C;
  double* sihc = s_dyn + 3 * (size_t)C;
  double* shf = s_dyn + 4 * (size_t)C;
  int* shn = (int*)(s_dyn + (4 + (size_t)F) * C);

  const double* __restrict__ hc = a.hcoef;
  const double* __restrict__ ihc = a.ihcoef;
  const double* __restrict__ hf = a.hf;
  const int* __restrict__ hn = a.hn;
  double* __restrict__ x = a.x;
  double* __restrict__ r = a.r;
  double* __restrict__ rt = a.rt;
  double* __restrict__ z = a.z;
  // the constant coefficients of cell j (owned by this CTA when SM)
  auto HC = [&](int j) { return SM ? shc[j - lo] : hc[j]; };
  auto IHC = [&](int j) { return SM ? sihc[j - lo] : ihc[j]; };
  auto HF = [&](int f, int j) { return SM ? shf[(size_t)f * C + (j - lo)] : hf[(size_t)f * nc + j]; };
  auto HN = [&](int f, int j) { return SM ? shn[(size_t)f * C + (j - lo)] : hn[(size_t)f * nc + j]; };

  // S1: coefficients (HCoefficients), lift setup x = 0 inside, x = h at type-3
  for (int j = lo + tid; j < hi; j += kHBlock) {
    double cf = a.Ac[j];
    for (int f = 0; f < F; ++f) {
      const int nb = a.nbr[j * F + f];
      const size_t o = (size_t)f * nc + j;
      double fc = 0.0;
      int nn = j;
      if (nb >= 0) {
        const int e = a.fedge[j * F + f];
        fc = a.tmp * a.D[e] * a.df[e] / a.dg[e];
        nn = nb;
        cf += fc;
      }
      a.hf[o] = fc;
      a.hn[o] = nn;
      if (SM) {
        shf[(size_t)f * C + (j - lo)] = fc;
        shn[(size_t)f * C + (j - lo)] = nn;
      }
    }
    a.hcoef[j] = cf;
    if (HP == 1) a.ihcoef[j] = 1.0 / cf;
    if (SM) {
      shc[j - lo] = cf;
      if (HP == 1) sihc[j - lo] = 1.0 / cf;
    }
    a.x[j] = 0.0;
    a.p[j] = a.b_in[j];
    a.p1[j] = 0.0;
  }
  for (int j = nc + blockIdx.x * kHBlock + tid; j < a.ncells; j += G * kHBlock) {
    a.x[j] = a.h_in[j];
    a.p[j] = 0.0;  // b = 0 at type-3 cells (3129-3134), and p stays 0 there
    a.p1[j] = 0.0;
    a.r[j] = 0.0;  // s = 0 outside the computational cells, so the direction
    a.rt[j] = 0.0; // formed for a neighbour there is 0, as p(bdy) = 0 (3134)
  }
  if (!grid_wait(ctl, ++nbar * G, 1)) return;

  // S2: z = A x; b -= z; r = b; s = M^-1 r; alpha0, eps0.  p1 (all zero) is the
  // first iteration's p_old, so that p = s + 0*p_old = s (3138-3147).
  // Thread 0 keeps the scalar state; the others read mu, nu, done from s_sc.
  double alpha = 0.0, eps = 0.0, eps0 = 0.0, mu_t = 0.0;
  int n = 0, status = SGPU_OK;
  {
    double part[2] = {0.0, 0.0};
    for (int j = lo + tid; j < hi; j += kHBlock) {
      double y = HC(j) * x[j];
      for (int f = 0; f < F; ++f) y -= HF(f, j) * x[HN(f, j)];
      const double rj = a.p[j] - y;
      r[j] = rj;
      if (HP == 1) {
        const double sj = rj * IHC(j);
        rt[j] = sj;
        part[0] += rj * sj;
        part[1] += rj * rj;
      } else {
        part[0] += rj * rj;
      }
    }
    cta_sum<2, kHBlock>(part, s_red);
    if (tid == 0) {
      partB[blockIdx.x] = part[0];
      partB[G + blockIdx.x] = part[1];
    }
    if (!grid_wait(ctl, ++nbar * G, 2)) return;
    grid_sum<2>(partB, G, [&](const double* tot) {
      alpha = tot[0];
      double alpha0 = tot[0];
      if (!a.resnorm) alpha0 = 1;
      if (HP == 1) eps = eps0 = tot[1];
      else eps = eps0 = alpha0;
      s_sc[0] = 0.0;  // mu of the first direction
      s_sc[2] = (a.maxiters <= 0 || eps == 0 || alpha == 0) ? 1.0 : 0.0;
    });
  }

  const double* __restrict__ sv = (HP == 1) ? a.rt : a.r;
  for (;;) {
    if (s_sc[2] != 0.0) break;
    const double mu = s_sc[0];
    // p_old of iteration n is p1 for even n, p for odd n; p_new the other one
    const double* __restrict__ po = (n & 1) ? a.p : a.p1;
    double* __restrict__ pn = (n & 1) ? a.p1 : a.p;
    phase_mark(ctl, 0);
    // A: p = s + mu p_old (own cells and neighbours), z = A p, p.z
    double pz = 0.0;
    if (SM) {
      cells2(lo + tid, hi, kHBlock, [&](int j0, int j1, bool two) {
        const double p0 = hdir(sv, po, mu, j0), p1 = hdir(sv, po, mu, j1);
        sp[j0 - lo] = p0;
        pn[j0] = p0;
        if (two) {
          sp[j1 - lo] = p1;
          pn[j1] = p1;
        }
      });
      __syncthreads();
      cells2(lo + tid, hi, kHBlock, [&](int j0, int j1, bool two) {
        const double p0 = sp[j0 - lo], p1 = sp[j1 - lo];
        double y0 = HC(j0) * p0, y1 = HC(j1) * p1;
        for (int f = 0; f < F; ++f) {
          const int k0 = HN(f, j0), k1 = HN(f, j1);
          const double w0 = HF(f, j0), w1 = HF(f, j1);
          const double q0 = (k0 >= lo && k0 < hi) ? sp[k0 - lo] : hdir(sv, po, mu, k0);
          const double q1 = (k1 >= lo && k1 < hi) ? sp[k1 - lo] : hdir(sv, po, mu, k1);
          y0 = __fma_rn(-w0, q0, y0);
          y1 = __fma_rn(-w1, q1, y1);
        }
        sz[j0 - lo] = y0;
        pz = __fma_rn(p0, y0, pz);
        if (two) {
          sz[j1 - lo] = y1;
          pz = __fma_rn(p1, y1, pz);
        }
      });
    } else {
      cells2(lo + tid, hi, kHBlock, [&](int j0, int j1, bool two) {
        const double p0 = hdir(sv, po, mu, j0), p1 = hdir(sv, po, mu, j1);
        double y0 = hc[j0] * p0, y1 = hc[j1] * p1;
        for (int f = 0; f < F; ++f) {
          const size_t o0 = (size_t)f * nc + j0, o1 = (size_t)f * nc + j1;
          const int k0 = hn[o0], k1 = hn[o1];
          const double w0 = hf[o0], w1 = hf[o1];
          y0 = __fma_rn(-w0, hdir(sv, po, mu, k0), y0);
          y1 = __fma_rn(-w1, hdir(sv, po, mu, k1), y1);
        }
        pn[j0] = p0;
        z[j0] = y0;
        pz = __fma_rn(p0, y0, pz);
        if (two) {
          pn[j1] = p1;
          z[j1] = y1;
          pz = __fma_rn(p1, y1, pz);
        }
      });
    }
    phase_mark(ctl, 7);
    {
      double part[1] = {pz};
      cta_sum<1, kHBlock>(part, s_red);
      if (tid == 0) partA[(n & 1) * G + blockIdx.x] = part[0];
    }
    if (!grid_wait(ctl, ++nbar * G, 3)) return;
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
    const double nu = s_sc[1];
    phase_mark(ctl, 5);
    // B: x += nu p; r -= nu z; s = M^-1 r; r.s, r.r
    double rs = 0.0, rr = 0.0;
    cells2(lo + tid, hi, kHBlock, [&](int j0, int j1, bool two) {
      const double pa = SM ? sp[j0 - lo] : pn[j0], pb = SM ? sp[j1 - lo] : pn[j1];
      const double za = SM ? sz[j0 - lo] : z[j0], zb = SM ? sz[j1 - lo] : z[j1];
      // one explicit FMA per update and inner-product term (FP64-pipe bound)
      const double ra = __fma_rn(-nu, za, r[j0]), rb = __fma_rn(-nu, zb, r[j1]);
      const double xa = __fma_rn(nu, pa, x[j0]), xb = __fma_rn(nu, pb, x[j1]);
      double sa = 0.0, sb = 0.0;
      if (HP == 1) {
        sa = ra * IHC(j0);
        sb = rb * IHC(j1);
      }
      x[j0] = xa;
      r[j0] = ra;
      if (HP == 1) {
        rt[j0] = sa;
        rs = __fma_rn(ra, sa, rs);
        rr = __fma_rn(ra, ra, rr);
      } else {
        rs = __fma_rn(ra, ra, rs);
      }
      if (two) {
        x[j1] = xb;
        r[j1] = rb;
        if (HP == 1) {
          rt[j1] = sb;
          rs = __fma_rn(rb, sb, rs);
          rr = __fma_rn(rb, rb, rr);
        } else {
          rs = __fma_rn(rb, rb, rs);
        }
      }
    });
    phase_mark(ctl, 6);
    double part[2] = {rs, rr};
    cta_sum<2, kHBlock>(part, s_red);
    if (tid == 0) {
      partB[(size_t)(n & 1) * 2 * G + blockIdx.x] = part[0];
      partB[(size_t)(n & 1) * 2 * G + G + blockIdx.x] = part[1];
    }
    if (!grid_wait(ctl, ++nbar * G, 4)) return;
    grid_sum<2>(partB + (size_t)(n & 1) * 2 * G, G, [&](const double* tot) {
      alpha = tot[0];
      mu_t *= alpha;
      eps = (HP == 1) ? tot[1] : alpha;
      const bool conv = sqrt(eps / eps0) < a.epsilon;
      s_sc[0] = mu_t;
      double done = 0.0;
      if (!isfinite(alpha)) {
        status = SGPU_BREAKDOWN;
        done = 1.0;
      } else if (conv || eps == 0 || alpha == 0) {
        done = 1.0;
      } else if (n + 1 >= a.maxiters) {
        status = SGPU_MAXITER;
        done = 1.0;
      }
      s_sc[2] = done;
    });
    ++n;
  }
  if (blockIdx.x == 0 && tid == 0) {
    ctl->alpha = alpha;
    ctl->eps = eps;
    ctl->eps0 = eps0;
    ctl->mu = mu_t;
    ctl->n = n;
    if (status != SGPU_OK) atomicCAS(&ctl->status, SGPU_OK, status);
    ctl->done = 1;
  }
}

int h_block() { return kHBlock; }

template <int HP, bool SM>
static const void* h_fn() {
  return (const void*)cgsolve_kernel<HP, SM>;
}

int h_max_grid(int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const void* fns[4] = {h_fn<0, false>(), h_fn<1, false>(), h_fn<0, true>(), h_fn<1, true>()};
  int per = 1 << 20;
  for (int k = 0; k < 4; ++k) {
    const size_t dyn = k < 2 ? 0 : kHMaxDynSmem;
    if (k >= 2 && cudaFuncSetAttribute(fns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
      return 0;
    int q = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, fns[k], kHBlock, dyn) != cudaSuccess) return 0;
    per = q < per ? q : per;
  }
  return sms * per;
}

cudaError_t h_launch(const HArgs& a, int grid, cudaStream_t st) {
  void* args[] = {(void*)&a};
  const size_t dyn = (size_t)a.cpc * (sizeof(double) * (4 + a.F) + sizeof(int) * a.F);
  const bool sm = dyn <= kHMaxDynSmem;
  const void* fn = a.hprecond == 1 ? (sm ? h_fn<1, true>() : h_fn<1, false>())
                                   : (sm ? h_fn<0, true>() : h_fn<0, false>());
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kHBlock), args, sm ? dyn : 0, st);
}

}  // namespace sgpu
