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
// (about 100 bytes per cell) stays in L2 for up to ~1M cells; this kernel is
// bound by its three grid barriers per iteration, not by HBM.
#include "sgpu_common.cuh"
#include "sgpu_q.h"

namespace sgpu {

__device__ __forceinline__ double h_apply(const HArgs& a, const double* xin, int j) {
  double y = a.hcoef[j] * xin[j];
  for (int f = 0; f < a.F; ++f) {
    const size_t o = (size_t)f * a.ncomp + j;
    y -= a.hf[o] * xin[a.hn[o]];
  }
  return y;
}

__global__ void __launch_bounds__(kBlock) cgsolve_kernel(HArgs a) {
  __shared__ double s_red[4 * (kBlock / 32)];
  SolveCtl* ctl = a.ctl;
  const int G = gridDim.x;
  const int tid = threadIdx.x;
  const int stride = G * kBlock;
  const int gid = blockIdx.x * kBlock + tid;

  // S1: coefficients (HCoefficients), lift setup x = 0 inside, x = h at type-3
  for (int j = gid; j < a.ncomp; j += stride) {
    double cf = a.Ac[j];
    for (int f = 0; f < a.F; ++f) {
      const int nb = a.nbr[j * a.F + f];
      const size_t o = (size_t)f * a.ncomp + j;
      if (nb >= 0) {
        const int e = a.fedge[j * a.F + f];
        const double fc = a.tmp * a.D[e] * a.df[e] / a.dg[e];
        a.hf[o] = fc;
        a.hn[o] = nb;
        cf += fc;
      } else {
        a.hf[o] = 0.0;
        a.hn[o] = j;
      }
    }
    a.hcoef[j] = cf;
    a.x[j] = 0.0;
    a.p[j] = a.b_in[j];
    a.z[j] = 0.0;
    a.r[j] = 0.0;
    a.rt[j] = 0.0;
  }
  for (int j = a.ncomp + gid; j < a.ncells; j += stride) {
    a.x[j] = a.h_in[j];
    a.p[j] = 0.0;  // b = 0 at type-3 cells (3129-3134)
  }
  if (!grid_sync(ctl, 1, [] {})) return;

  // S2: z = A x; b -= z; r = b; preconditioned start; alpha0, eps0
  {
    double part[2] = {0.0, 0.0};
    for (int j = gid; j < a.ncomp; j += stride) {
      const double zj = h_apply(a, a.x, j);
      const double pj = a.p[j] - zj;
      a.r[j] = pj;
      if (a.hprecond == 1) {
        const double rtj = pj / a.hcoef[j];
        a.rt[j] = rtj;
        a.p[j] = rtj;
        part[0] += pj * rtj;
        part[1] += pj * pj;
      } else {
        a.p[j] = pj;
        part[0] += pj * pj;
      }
    }
    block_sum<2>(part, s_red);
    if (tid == 0) {
      a.partials[blockIdx.x] = part[0];
      a.partials[G + blockIdx.x] = part[1];
    }
    if (!grid_sync(ctl, 2, [&] {
          double tot[2];
          reduce_partials<2>(a.partials, G, G, tot, s_red);
          if (tid == 0) {
            double alpha = tot[0], alpha0 = tot[0];
            if (!a.resnorm) alpha0 = 1;
            double eps, eps0;
            if (a.hprecond == 1) eps = eps0 = tot[1];
            else eps = eps0 = alpha0;
            ctl->alpha = alpha;
            ctl->alpha0 = alpha0;
            ctl->eps = eps;
            ctl->eps0 = eps0;
            ctl->n = 0;
            ctl->done = (a.maxiters <= 0 || eps == 0 || alpha == 0) ? 1 : 0;
            __threadfence();
          }
        }))
      return;
  }

  for (;;) {
    if (ld_volatile_int(&ctl->done)) break;
    {
      double part[1] = {0.0};
      for (int j = gid; j < a.ncomp; j += stride) {
        const double zj = h_apply(a, a.p, j);
        a.z[j] = zj;
        part[0] += a.p[j] * zj;
      }
      block_sum<1>(part, s_red);
      if (tid == 0) a.partials[blockIdx.x] = part[0];
      if (!grid_sync(ctl, 3, [&] {
            double tot[1];
            reduce_partials<1>(a.partials, G, G, tot, s_red);
            if (tid == 0) {
              const double alpha = *(volatile double*)&ctl->alpha;
              ctl->mu = 1 / alpha;
              const double nu = alpha / tot[0];
              ctl->nu = nu;
              if (!isfinite(nu)) {
                ctl->status = SGPU_BREAKDOWN;
                ctl->done = 1;
              }
              __threadfence();
            }
          }))
        return;
      if (ld_volatile_int(&ctl->done)) break;
    }
    {
      const double nu = *(volatile double*)&ctl->nu;
      double part[2] = {0.0, 0.0};
      for (int j = gid; j < a.ncomp; j += stride) {
        a.x[j] += nu * a.p[j];
        const double rj = a.r[j] - nu * a.z[j];
        a.r[j] = rj;
        if (a.hprecond == 1) {
          const double rtj = rj / a.hcoef[j];
          a.rt[j] = rtj;
          part[0] += rj * rtj;
          part[1] += rj * rj;
        } else {
          part[0] += rj * rj;
        }
      }
      block_sum<2>(part, s_red);
      if (tid == 0) {
        a.partials[blockIdx.x] = part[0];
        a.partials[G + blockIdx.x] = part[1];
      }
      if (!grid_sync(ctl, 4, [&] {
            double tot[2];
            reduce_partials<2>(a.partials, G, G, tot, s_red);
            if (tid == 0) {
              const double alpha = tot[0];
              double mu = *(volatile double*)&ctl->mu;
              mu *= alpha;
              ctl->mu = mu;
              ctl->alpha = alpha;
              const double eps = (a.hprecond == 1) ? tot[1] : alpha;
              ctl->eps = eps;
              const int n = ctl->n + 1;
              ctl->n = n;
              const double eps0 = ctl->eps0;
              int done = 0;
              const bool conv = sqrt(eps / eps0) < a.epsilon;
              if (conv || n >= a.maxiters || eps == 0 || alpha == 0) done = 1;
              if (!isfinite(alpha)) {
                ctl->status = SGPU_BREAKDOWN;
                done = 1;
              }
              if (done && !conv && n >= a.maxiters && ctl->status == SGPU_OK) ctl->status = SGPU_MAXITER;
              ctl->done = done;
              __threadfence();
            }
          }))
        return;
      if (ld_volatile_int(&ctl->done)) break;
    }
    {
      const double mu = *(volatile double*)&ctl->mu;
      const double* src = (a.hprecond == 1) ? a.rt : a.r;
      for (int j = gid; j < a.ncomp; j += stride) a.p[j] = src[j] + mu * a.p[j];
      if (!grid_sync(ctl, 5, [] {})) return;
    }
  }
}

int h_max_grid(int device) {
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cgsolve_kernel, kBlock, 0) != cudaSuccess)
    return 0;
  return sms * per;
}

cudaError_t h_launch(const HArgs& a, int grid, cudaStream_t st) {
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)cgsolve_kernel, dim3(grid), dim3(kBlock), args, 0, st);
}

}  // namespace sgpu
