// sgpu_step.cu -- the steps on either side of CGSolveQ in SUNTANS's Solve
// (main/phys.c:1273-1287), and the per-step refresh of the vertical grid that
// drives both solvers' coefficients, on the device:
//
//   ComputeQSource  main/phys.c:2345-2395  src = div(u*, w*) / dt, D = df/dg
//   Corrector       main/phys.c:2301-2333  u -= dt/dg grad(qc), w from the
//                                          vertical gradient of qc, q += qc
//   UpdateDZ        main/phys.c:816-941    dzz, ctop, etop from the free surface
//                                          (option 0, the per-step call)
//   SetFluxHeight   main/phys.c:4338-4435  dzf from u, dzz and h
//
// Layout (device order of sgpu_api.cu): cell columns j in cellp order, slots
// [dcoff[j], dcoff[j] + Nk); w-like fields with Nk + 1 levels per column at
// [woff[j], woff[j] + Nk + 1); edge fields (u, utmp2, dzf) in edge order at
// [eoff[e], eoff[e] + Nke[e]).  Every floating-point expression is evaluated
// in the reference's order with explicitly rounded operations (no contraction
// into FMA), so the results are the reference's bits.
#include "sgpu_step.h"

namespace sgpu {

// src at every slot (computational slots from the divergence, 0 elsewhere).
__global__ void qsource_kernel(StepArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n3; u += T) {
    if (u >= a.n3c) {
      a.src[u] = 0.0;
      continue;
    }
    const int j = a.slotcol[u];
    const int k = u - a.dcoff[j];
    const int ctop = a.ctop[j];
    if (k < ctop) {
      a.src[u] = 0.0;
      continue;
    }
    // vertical contribution (2369-2373)
    const double Ac = a.Ac[j];
    const int wo = a.woff[j] + k;
    double s = __dadd_rn(__dmul_rn(Ac, __dsub_rn(a.w[wo], a.w[wo + 1])),
                         __dmul_rn(__dmul_rn(a.thetafactor, Ac), __dsub_rn(a.wtmp2[wo], a.wtmp2[wo + 1])));
    // horizontal contributions, face by face (2377-2386)
    for (int f = 0; f < a.nfaces[j]; ++f) {
      const int ne = a.fedge[j * a.F + f];
      if (k >= a.nke[ne]) continue;
      const int eo = a.eoff[ne] + k;
      const double flux = __dadd_rn(a.u[eo], __dmul_rn(a.thetafactor, a.utmp2[eo]));
      s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(flux, a.dzf[eo]), (double)a.normal[j * a.F + f]), a.df[ne]));
    }
    a.src[u] = __ddiv_rn(s, a.dt);  // 2389-2390
  }
  // D = df/dg on every edge (2392-2394)
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.Ne; e += T) a.D[e] = __ddiv_rn(a.df[e], a.dg[e]);
}

// u on the computational edges (2306-2312): one thread per edge.
__global__ void corrector_edges_kernel(StepArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.ncedge; t += T) {
    const int e = a.cedge[t];
    const int top = a.etop[e], nke = a.nke[e];
    if (!(a.D[e] != 0.0 && top < nke - 1)) continue;
    const int o0 = a.dcoff[a.grad[2 * e]], o1 = a.dcoff[a.grad[2 * e + 1]];
    const double f = __ddiv_rn(a.dt, a.dg[e]);
    for (int k = top; k < nke; ++k) {
      const int eo = a.eoff[e] + k;
      a.u_out[eo] = __dsub_rn(a.u_out[eo], __dmul_rn(f, __dsub_rn(a.qc[o0 + k], a.qc[o1 + k])));
    }
  }
}

// w and q on the computational columns (2315-2331): one thread per column.
__global__ void corrector_cells_kernel(StepArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.ncomp; j += T) {
    const int ctop = a.ctop[j], nk = a.nk[j], o = a.dcoff[j], wo = a.woff[j];
    const double dt2 = __dmul_rn(2.0, a.dt);
    for (int k = ctop + 1; k < nk; ++k)
      a.w_out[wo + k] = __dsub_rn(a.w_out[wo + k], __dmul_rn(__ddiv_rn(dt2, __dadd_rn(a.dzz[o + k - 1], a.dzz[o + k])),
                                                              __dsub_rn(a.qc[o + k - 1], a.qc[o + k])));
    a.w_out[wo + ctop] = __dadd_rn(a.w_out[wo + ctop], __dmul_rn(__ddiv_rn(dt2, a.dzz[o + ctop]), a.qc[o + ctop]));
    if (ctop < nk - 1)
      for (int k = ctop; k < nk; ++k) a.q_out[o + k] = __dadd_rn(a.q_out[o + k], a.qc[o + k]);
  }
}

// ---------------------------------------------------------------------------
// UpdateDZ, option 0 (main/phys.c:816-941) and SetFluxHeight (4338-4435)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ref_max(double x1, double x2) { return x2 > x1 ? x2 : x1; }  // util.c:212
__device__ __forceinline__ double ref_min(double x, double y) { return x < y ? x : y; }        // util.c:242
__device__ __forceinline__ double upwind(double u, double dz1, double dz2) {                 // util.c:219
  if (fabs(u) > 0) return u > 0 ? dz2 : dz1;
  return ref_max(dz1, dz2);
}

// one thread per cell: save the old state, then the new dzz and ctop from h
__global__ void update_dz_cells_kernel(VGridArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.Nc; j += T) {
    const int o = a.dcoff[j], nk = a.nk[j], ct = a.ctop[j];
    const double dv = a.dv[j], h = a.h[j];
    a.ctopold[j] = ct;
    for (int k = 0; k < ct; ++k) a.dzzold[o + k] = 0;
    for (int k = ct; k < nk; ++k) a.dzzold[o + k] = a.dzz[o + k];
    double z = 0;
    for (int k = 0; k < nk; ++k) z = __dsub_rn(z, a.dz[k]);
    a.dzz[o + nk - 1] = __dadd_rn(__dadd_rn(a.dz[nk - 1], dv), z);
    if (a.Nkmax > 1) {
      int ctop = ct, flag = 0;
      z = 0;
      for (int k = 0; k < nk; ++k) {
        z = __dsub_rn(z, a.dz[k]);
        double v;
        if (h >= z) {
          if (!flag) {
            if (k == nk - 1) {
              v = __dadd_rn(h, dv);
              ctop = k;
            } else if (h == z) {
              v = 0;
              ctop = k + 1;
            } else {
              v = __dsub_rn(h, z);
              ctop = k;
            }
            flag = 1;
          } else {
            if (k == nk - 1) v = __dadd_rn(__dadd_rn(a.dz[k], dv), z);
            else if (z < -dv) v = 0;
            else v = a.dz[k];
          }
        } else {
          v = 0;
        }
        a.dzz[o + k] = v;
      }
      a.ctop[j] = ctop;
    } else {
      a.dzz[o] = __dadd_rn(dv, h);
    }
  }
}

// one thread per edge: etopold, then etop from the new ctop (903-914)
__global__ void update_dz_edges_kernel(VGridArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.Ne; e += T) {
    a.etopold[e] = a.etop[e];
    const int n1 = a.grad[2 * e], n2 = a.grad[2 * e + 1];
    int t;
    if (n1 == -1) t = a.ctop[n2];
    else if (n2 == -1) t = a.ctop[n1];
    else t = a.ctop[n1] < a.ctop[n2] ? a.ctop[n1] : a.ctop[n2];
    a.etop[e] = t;
  }
}

// the bottom level of every cell: pass 0 before the fluxes (4386-4392),
// pass 1 after them (4430-4433); only when smoothbot != 0
__global__ void smoothbot_kernel(VGridArgs a, int pass) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.Nc; j += T) {
    const int nk = a.nk[j], u = a.dcoff[j] + nk - 1;
    if (pass == 0) a.dzz[u] = ref_max(a.dzbot[j], __dmul_rn(a.smoothbot, a.dz[nk - 1]));
    else a.dzz[u] = ref_max(a.dzz[u], __dmul_rn(a.dzsmall, a.dz[nk - 1]));
  }
}

// one thread per edge: the flux heights of its levels (4395-4426)
__global__ void flux_height_kernel(VGridArgs a) {
  const int T = gridDim.x * blockDim.x;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.Ne; e += T) {
    int n1 = a.grad[2 * e], n2 = a.grad[2 * e + 1];
    if (n1 == -1) n1 = n2;
    if (n2 == -1) n2 = n1;
    const int eo = a.eoff[e], top = a.etop[e], nke = a.nke[e];
    const int o1 = a.dcoff[n1], o2 = a.dcoff[n2];
    for (int k = 0; k < top && k < nke; ++k) a.dzf[eo + k] = 0;
    for (int k = top; k < nke; ++k) a.dzf[eo + k] = upwind(a.u[eo + k], a.dzz[o1 + k], a.dzz[o2 + k]);
    if (nke < 1) continue;
    const int k = nke - 1;
    if (top == k)
      a.dzf[eo + k] = ref_max(0, __dadd_rn(upwind(a.u[eo + k], a.h[n1], a.h[n2]), ref_min(a.dv[n1], a.dv[n2])));
    else
      a.dzf[eo + k] = ref_min(a.dzz[o1 + k], a.dzz[o2 + k]);
    for (int kk = top; kk < nke; ++kk)
      if (a.dzf[eo + kk] <= 1e-10) a.dzf[eo + kk] = 0;  // DRYCELLHEIGHT, suntans.h:31
  }
}

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)std::max(1LL, std::min(g, 152LL * 16));
}

cudaError_t launch_qsource(const StepArgs& a, cudaStream_t st) {
  qsource_kernel<<<grid_for(std::max<long long>(a.n3, a.Ne)), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_update_dz(const VGridArgs& a, cudaStream_t st) {
  update_dz_cells_kernel<<<grid_for(a.Nc), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  update_dz_edges_kernel<<<grid_for(a.Ne), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_set_flux_height(const VGridArgs& a, cudaStream_t st) {
  cudaError_t e;
  if (a.smoothbot != 0) {
    smoothbot_kernel<<<grid_for(a.Nc), 256, 0, st>>>(a, 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  flux_height_kernel<<<grid_for(a.Ne), 256, 0, st>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (a.smoothbot != 0) {
    smoothbot_kernel<<<grid_for(a.Nc), 256, 0, st>>>(a, 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_corrector(const StepArgs& a, cudaStream_t st) {
  corrector_edges_kernel<<<grid_for(a.ncedge), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  corrector_cells_kernel<<<grid_for(a.ncomp), 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sgpu
