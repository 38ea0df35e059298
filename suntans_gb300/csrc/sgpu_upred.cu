// sgpu_upred.cu -- UPredictor (main/phys.c:2579-3077) on the device: the
// vertically implicit predictor of the horizontal velocity, the free-surface
// right-hand side that CGSolve reads, and the velocity update after it.
//
//   upred_vertical   2626-2945  per computational edge: the explicit free-surface
//                               gradient, wind stress, viscous and vertical
//                               advection terms, then two Thomas solves for
//                               U*** = A^{-1} U** and E = A^{-1} [1..1], and
//                               D = dzf^T E; one thread per edge, its columns in
//                               thread-local memory
//   upred_rhs        2964-2977  per computational cell: htmp = Ac h - dt sum of
//                               the face fluxes ((1-theta) u + theta U***) df dzf
//   upred_velocity   2991-3019  dry-cell clip of h, u = U*** - g theta dt E dh/dg
//   upred_boundary   3046-3076  u on type-2 edges and on the mark-3 faces of
//                               type-3 cells (continuity)
//
// Every expression is evaluated in the reference's order with explicitly
// rounded operations (no contraction into FMA), so the results are the
// reference's bits.  One difference: with a no-slip top or bottom on a
// single-layer edge the reference reads c[Nke] (2864-2871), a scratch value
// that an earlier edge left behind; here that value is 0.
#include "sgpu_step.h"

namespace sgpu {

namespace {
__device__ __forceinline__ double ADD(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ double SUB(double x, double y) { return __dsub_rn(x, y); }
__device__ __forceinline__ double MUL(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ double DIV(double x, double y) { return __ddiv_rn(x, y); }

// TriSolve, main/util.c:185-203 (a, b, c, d modified; u written)
__device__ void thomas_rn(double* a, double* b, double* c, double* d, double* u, int N) {
  for (int k = 1; k < N; ++k) {
    b[k] = SUB(b[k], DIV(MUL(a[k], c[k - 1]), b[k - 1]));
    d[k] = SUB(d[k], DIV(MUL(a[k], d[k - 1]), b[k - 1]));
  }
  u[N - 1] = DIV(d[N - 1], b[N - 1]);
  for (int k = N - 2; k >= 0; --k) u[k] = SUB(DIV(d[k], b[k]), DIV(MUL(c[k], u[k + 1]), b[k]));
}
}  // namespace

template <int KMAX>
__global__ void __launch_bounds__(128) upred_vertical_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A.ncedge; t += T) {
    const int j = A.cedge[t];
    const int c1 = A.grad[2 * j], c2 = A.grad[2 * j + 1];
    const int et = A.etop[j], nk = A.nke[j], eo = A.eoff[j];
    double* ut = A.utmp + eo;
    const double* uu = A.u + eo;
    // the old free-surface gradient (2626-2635), with the model's theta
    {
      const double g = DIV(MUL(MUL(MUL(A.grav, SUB(1.0, A.theta)), A.dt), SUB(A.h[c1], A.h[c2])), A.dg[j]);
      for (int k = et; k < nk; ++k) ut[k] = SUB(ut[k], g);
    }
    const double dt = A.dt, theta = 1.0, alpha = 1.0;  // drag fully implicit (2637-2646)
    const double* z1 = A.dzz + A.dcoff[c1];
    const double* z2 = A.dzz + A.dcoff[c2];
    double a[KMAX], b[KMAX], c[KMAX], d[KMAX], e1[KMAX], a0[KMAX], b0[KMAX], c0[KMAX];
    ut[et] = ADD(ut[et], DIV(MUL(MUL(2.0, dt), A.tau_T[j]), ADD(z1[et], z2[et])));  // 2662-2663
    if (z1[et] == 0 && z2[et] == 0) continue;                                       // 2667
    for (int k = et; k < nk; ++k) a[k] = b[k] = c[k] = d[k] = 0;
    c[nk] = 0;
    {
      const double* t1 = A.nu_tv + A.dcoff[c1];
      const double* t2 = A.nu_tv + A.dcoff[c2];
      const double* l1 = A.nu_lax + A.dcoff[c1];
      const double* l2 = A.nu_lax + A.dcoff[c2];
      for (int k = et + 1; k < nk; ++k)  // 2679-2683
        c[k] = MUL(0.25, ADD(ADD(ADD(ADD(t1[k - 1], t2[k - 1]), t1[k]), t2[k]),
                             MUL(A.lax, ADD(ADD(ADD(l1[k - 1], l2[k - 1]), l1[k]), l2[k]))));
    }
    for (int k = et + 1; k < nk; ++k)  // 2687-2690
      a[k] = DIV(MUL(2.0, ADD(A.nu, c[k])),
                 MUL(MUL(0.25, ADD(z1[k], z2[k])), ADD(ADD(ADD(z1[k - 1], z2[k - 1]), z1[k]), z2[k])));
    for (int k = et; k < nk - 1; ++k)  // 2692-2696
      b[k] = DIV(MUL(2.0, ADD(A.nu, c[k + 1])),
                 MUL(MUL(0.25, ADD(z1[k], z2[k])), ADD(ADD(ADD(z1[k], z2[k]), z1[k + 1]), z2[k + 1])));
    const bool adv = A.nonlinear && A.thetaM >= 0 && nk - et > 1;
    if (adv) {  // 2702-2723
      int n0, n1;
      if (A.ctop[c1] > A.ctop[c2]) {
        n0 = c2;
        n1 = c1;
      } else {
        n0 = c1;
        n1 = c2;
      }
      const int ct = A.ctop[n1];
      const double* w0 = A.w + A.woff[n0];
      const double* w1 = A.w + A.woff[n1];
      for (int k = 0; k < ct && k < KMAX; ++k) d[k] = 0;
      for (int k = ct; k < nk; ++k) d[k] = MUL(0.5, ADD(w0[k], w1[k]));
      d[nk] = 0;
      for (int k = et; k < nk; ++k) {
        const double den = MUL(0.5, ADD(z1[k], z2[k]));
        a0[k] = DIV(ADD(MUL(MUL(alpha, 0.5), SUB(d[k], fabs(d[k]))), MUL(MUL(0.5, SUB(1.0, alpha)), d[k])), den);
        b0[k] = DIV(ADD(MUL(MUL(alpha, 0.5), ADD(SUB(ADD(d[k], fabs(d[k])), d[k + 1]), fabs(d[k + 1]))),
                        MUL(MUL(0.5, SUB(1.0, alpha)), SUB(d[k], d[k + 1]))),
                    den);
        c0[k] = DIV(-ADD(MUL(MUL(alpha, 0.5), ADD(d[k + 1], fabs(d[k + 1]))), MUL(MUL(0.5, SUB(1.0, alpha)), d[k + 1])),
                    den);
      }
    }
    const double ex = MUL(dt, SUB(1.0, theta));  // dt*(1-theta)
    const double CdT = A.CdT[j], CdB = A.CdB[j];
    if (nk - et > 1) {  // 2726-2771
      for (int k = et + 1; k < nk - 1; ++k)
        ut[k] = ADD(ut[k], MUL(ex, ADD(SUB(MUL(a[k], uu[k - 1]), MUL(ADD(a[k], b[k]), uu[k])), MUL(b[k], uu[k + 1]))));
      if (CdT == -1)
        ut[et] = ADD(ut[et], MUL(ex, ADD(SUB(MUL(a[et], -uu[et]), MUL(ADD(a[et], b[et]), uu[et])),
                                         MUL(b[et], uu[et + 1]))));
      else
        ut[et] = ADD(ut[et],
                     MUL(ex, ADD(MUL(-ADD(b[et], DIV(MUL(MUL(2.0, CdT), fabs(uu[et])), ADD(z1[et], z2[et]))), uu[et]),
                                 MUL(b[et], uu[et + 1]))));
      const int kb = nk - 1;
      if (CdB == -1)
        ut[kb] = ADD(ut[kb], MUL(ex, ADD(SUB(MUL(a[kb], uu[kb - 1]), MUL(ADD(a[kb], b[kb]), uu[kb])),
                                         MUL(b[kb], -uu[kb]))));
      else
        ut[kb] = ADD(ut[kb],
                     MUL(ex, SUB(MUL(a[kb], uu[kb - 1]),
                                 MUL(ADD(a[kb], DIV(MUL(MUL(2.0, CdB), fabs(uu[kb])), ADD(z1[kb], z2[kb]))), uu[kb]))));
    } else {  // 2772-2798, with k == et (c[et] == 0)
      const double s = ADD(z1[et], z2[et]);
      const double ex2 = MUL(MUL(2.0, dt), SUB(1.0, theta));
      if (CdB == -1)
        ut[et] = SUB(ut[et], MUL(ex2, DIV(MUL(MUL(2.0, MUL(2.0, ADD(A.nu, c[et]))), uu[et]), MUL(s, s))));
      else
        ut[et] = SUB(ut[et], MUL(MUL(DIV(MUL(ex2, CdB), s), fabs(uu[et])), uu[et]));
      if (CdT == -1)
        ut[et] = SUB(ut[et], MUL(ex2, DIV(MUL(MUL(2.0, MUL(2.0, ADD(A.nu, c[et]))), uu[et]), MUL(s, s))));
      else
        ut[et] = SUB(ut[et], MUL(MUL(DIV(MUL(ex2, CdT), s), fabs(uu[et])), uu[et]));
    }
    if (adv) {  // 2801-2813
      const double em = MUL(A.dt, SUB(1.0, A.thetaM));
      for (int k = et + 1; k < nk - 1; ++k)
        ut[k] = SUB(ut[k], MUL(em, ADD(ADD(MUL(a0[k], uu[k - 1]), MUL(b0[k], uu[k])), MUL(c0[k], uu[k + 1]))));
      ut[et] = SUB(ut[et], MUL(em, ADD(MUL(ADD(a0[et], b0[et]), uu[et]), MUL(c0[et], uu[et + 1]))));
      const int kb = nk - 1;
      ut[kb] = SUB(ut[kb], MUL(em, ADD(MUL(a0[kb], uu[kb - 1]), MUL(ADD(b0[kb], c0[kb]), uu[kb]))));
    }
    for (int k = et; k < nk; ++k) {  // 2822-2825
      e1[k] = 1.0;
      d[k] = ut[k];
    }
    const double td = MUL(-theta, dt);  // -theta*dt
    const double tp = MUL(theta, dt);   // theta*dt
    if (nk - et > 1) {                  // 2827-2861
      c[et] = MUL(td, b[et]);
      if (CdT == -1)
        b[et] = ADD(1.0, MUL(tp, ADD(ADD(a[et], a[et + 1]), b[et])));
      else
        b[et] = ADD(1.0, MUL(tp, ADD(b[et], DIV(MUL(MUL(2.0, CdT), fabs(uu[et])), ADD(z1[et], z2[et])))));
      a[et] = 0;
      const int kb = nk - 1;
      c[kb] = 0;
      if (CdB == -1)
        b[kb] = ADD(1.0, MUL(tp, ADD(ADD(a[kb], b[kb]), b[kb - 1])));
      else
        b[kb] = ADD(1.0, MUL(tp, ADD(a[kb], DIV(MUL(MUL(2.0, CdB), fabs(uu[kb])), ADD(z1[kb], z2[kb])))));
      a[kb] = MUL(td, a[kb]);
      for (int k = et + 1; k < nk - 1; ++k) {
        c[k] = MUL(td, b[k]);
        b[k] = ADD(1.0, MUL(tp, ADD(a[k], b[k])));
        a[k] = MUL(td, a[k]);
      }
    } else {  // 2862-2887; c[nk] == 0 here (see the file comment)
      const double s = ADD(z1[et], z2[et]);
      const double t8 = MUL(MUL(MUL(4.0, theta), dt), 2.0);
      const double t2 = MUL(MUL(2.0, theta), dt);
      b[et] = 1.0;
      if (CdB == -1)
        b[et] = ADD(b[et], DIV(MUL(t8, ADD(A.nu, c[nk])), MUL(s, s)));
      else
        b[et] = ADD(b[et], MUL(DIV(MUL(t2, fabs(ut[et])), s), CdB));
      if (CdT == -1)
        b[et] = ADD(b[et], DIV(MUL(t8, ADD(A.nu, c[nk])), MUL(s, s)));
      else
        b[et] = ADD(b[et], MUL(DIV(MUL(t2, fabs(ut[et])), s), CdT));
    }
    if (adv) {  // 2890-2904
      const double pm = MUL(A.dt, A.thetaM);
      for (int k = et + 1; k < nk - 1; ++k) {
        a[k] = ADD(a[k], MUL(pm, a0[k]));
        b[k] = ADD(b[k], MUL(pm, b0[k]));
        c[k] = ADD(c[k], MUL(pm, c0[k]));
      }
      b[et] = ADD(b[et], MUL(pm, ADD(a0[et], b0[et])));
      c[et] = ADD(c[et], MUL(pm, c0[et]));
      const int kb = nk - 1;
      a[kb] = ADD(a[kb], MUL(pm, a0[kb]));
      b[kb] = ADD(b[kb], MUL(pm, ADD(b0[kb], c0[kb])));
    }
    double* E = A.E + eo;
    if (nk - et > 1) {  // 2922-2935
      for (int k = et; k < nk; ++k) {
        a0[k] = a[k];
        b0[k] = b[k];
        c0[k] = c[k];
      }
      thomas_rn(a + et, b + et, c + et, d + et, ut + et, nk - et);
      thomas_rn(a0 + et, b0 + et, c0 + et, e1 + et, E + et, nk - et);
    } else {
      ut[et] = DIV(ut[et], b[et]);
      E[et] = DIV(1.0, b[et]);
    }
    double Dj = 0;  // 2941-2943
    const double* zf = A.dzf + eo;
    for (int k = et; k < nk; ++k) Dj = ADD(Dj, MUL(E[k], zf[k]));
    A.D[j] = Dj;
  }
}

// D = 0 on every edge before the computational ones are written (2602-2603)
__global__ void upred_zero_d_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.Ne; e += T) A.D[e] = 0;
}

// NaN in U*** on any edge's wet levels (the reference stops, 2948-2954)
__global__ void upred_nan_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  int n = 0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.Ne; e += T) {
    const double* ut = A.utmp + A.eoff[e];
    for (int k = A.etop[e]; k < A.nke[e]; ++k) n += ut[k] != ut[k];
  }
  if (n) atomicAdd(A.nnan, n);
}

__global__ void upred_rhs_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  const double th = A.theta, om = SUB(1.0, A.theta);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.ncomp; j += T) {
    double sum = 0;
    for (int f = 0; f < A.nfaces[j]; ++f) {
      const int ne = A.fedge[j * A.F + f];
      const double nrm = (double)A.normal[j * A.F + f];
      const double dfe = A.df[ne];
      const int eo = A.eoff[ne];
      for (int k = A.etop[ne]; k < A.nke[ne]; ++k) {
        const double fl = ADD(MUL(om, A.u[eo + k]), MUL(th, A.utmp[eo + k]));
        sum = ADD(sum, MUL(MUL(MUL(fl, dfe), nrm), A.dzf[eo + k]));
      }
    }
    A.htmp[j] = SUB(MUL(A.Ac[j], A.h[j]), MUL(A.dt, sum));
  }
}

// OpenBoundaryFluxes without boundary data (boundaries.c:41-58): 0 n1 + 0 n2
__global__ void upred_open_fluxes_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A.nbnd; t += T) {
    const int j = A.bedge[t];
    const double v = ADD(MUL(0.0, A.n1[j]), MUL(0.0, A.n2[j]));
    double* ut = A.utmp + A.eoff[j];
    for (int k = A.etop[j]; k < A.nke[j]; ++k) ut[k] = v;
  }
}

__global__ void upred_dry_kernel(UPredArgs A) {  // 2993-3002
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.Nc; j += T) {
    const double lim = ADD(-A.dv[j], 1e-10);  // DRYCELLHEIGHT, main/suntans.h:31
    if (A.h[j] <= lim) {
      A.h[j] = lim;
      A.active[j] = 0;
    } else {
      A.active[j] = 1;
    }
  }
}

__global__ void upred_edge_velocity_kernel(UPredArgs A) {  // 3006-3019
  const int T = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A.ncedge; t += T) {
    const int j = A.cedge[t];
    const int c1 = A.grad[2 * j], c2 = A.grad[2 * j + 1];
    const int et = A.etop[j], nk = A.nke[j], eo = A.eoff[j];
    const double gtd = MUL(MUL(A.grav, A.theta), A.dt);
    const double dh = SUB(A.h[c1], A.h[c2]);
    for (int k = et; k < nk; ++k)
      A.u_out[eo + k] = SUB(A.utmp[eo + k], DIV(MUL(MUL(gtd, A.E[eo + k]), dh), A.dg[j]));
    if (et == nk - 1 && A.dzz[A.dcoff[c1] + et] == 0 && A.dzz[A.dcoff[c2] + et] == 0) A.u_out[eo + et] = 0;
  }
}

__global__ void upred_boundary_kernel(UPredArgs A) {  // 3046-3076
  const int T = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  for (int t = t0; t < A.nb2; t += T) {
    const int j = A.b2edge[t];
    const int eo = A.eoff[j];
    for (int k = A.etop[j]; k < A.nke[j]; ++k) A.u_out[eo + k] = A.utmp[eo + k];
  }
}

__global__ void upred_type3_kernel(UPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < A.ncell3; b += T) {
    const int nf = A.bnfaces[b];
    for (int f = 0; f < nf; ++f) {
      const int ne = A.bfedge[b * A.F + f];
      if (A.mark[ne] != 3) continue;
      const int eo = A.eoff[ne];
      const double nrm = (double)A.bnormal[b * A.F + f];
      for (int k = A.etop[ne]; k < A.nke[ne]; ++k) {
        A.u_out[eo + k] = 0;
        double sum = 0;
        for (int f1 = 0; f1 < nf; ++f1) {
          const int e1 = A.bfedge[b * A.F + f1];
          // levels past another face's row count as 0 (the reference reads past the row there)
          if (k < A.nke[e1])
            sum = ADD(sum, MUL(MUL(A.u_out[A.eoff[e1] + k], A.df[e1]), (double)A.bnormal[b * A.F + f1]));
        }
        A.u_out[eo + k] = DIV(DIV(-sum, A.df[ne]), nrm);
      }
    }
  }
}

static int blocks_for(long long n, int bs) {
  long long b = (n + bs - 1) / bs;
  return (int)std::max(1LL, std::min(b, 152LL * 16));
}

// one wave: every SM holds as many CTAs as fit, and the threads stride over
// the computational edges (sorted deepest first), so no partial second wave
// leaves SMs idle at the end
template <int KMAX>
static void vertical_launch(const UPredArgs& a, cudaStream_t st) {
  static int per_sm = -1, nsm = 0;
  if (per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, upred_vertical_kernel<KMAX>, 128, 0) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
  }
  const long long need = (a.ncedge + 127) / 128;
  const int nb = (int)std::max(1LL, std::min(need, (long long)per_sm * std::max(nsm, 1)));
  upred_vertical_kernel<KMAX><<<nb, 128, 0, st>>>(a);
}

cudaError_t launch_upred_vertical(const UPredArgs& a, cudaStream_t st) {
  upred_zero_d_kernel<<<blocks_for(a.Ne, 256), 256, 0, st>>>(a);
  if (a.ncedge > 0) {
    if (a.kmax <= 16) vertical_launch<16>(a, st);
    else if (a.kmax <= 32) vertical_launch<32>(a, st);
    else if (a.kmax <= 64) vertical_launch<64>(a, st);
    else vertical_launch<128>(a, st);
  }
  upred_nan_kernel<<<blocks_for(a.Ne, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_upred_rhs(const UPredArgs& a, cudaStream_t st) {
  if (a.ncomp > 0) upred_rhs_kernel<<<blocks_for(a.ncomp, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_upred_open_fluxes(const UPredArgs& a, cudaStream_t st) {
  if (a.nbnd > 0) upred_open_fluxes_kernel<<<blocks_for(a.nbnd, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_upred_velocity(const UPredArgs& a, cudaStream_t st) {
  upred_dry_kernel<<<blocks_for(a.Nc, 256), 256, 0, st>>>(a);
  if (a.ncedge > 0) upred_edge_velocity_kernel<<<blocks_for(a.ncedge, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_upred_boundary(const UPredArgs& a, cudaStream_t st) {
  if (a.nb2 > 0) upred_boundary_kernel<<<blocks_for(a.nb2, 256), 256, 0, st>>>(a);
  if (a.ncell3 > 0) upred_type3_kernel<<<blocks_for(a.ncell3, 128), 128, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sgpu
