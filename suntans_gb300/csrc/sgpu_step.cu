// sgpu_step.cu -- the steps on either side of CGSolveQ in SUNTANS's Solve
// (main/phys.c:1273-1287), on the device:
//
//   ComputeQSource  main/phys.c:2345-2395  src = div(u*, w*) / dt, D = df/dg
//   Corrector       main/phys.c:2301-2333  u -= dt/dg grad(qc), w from the
//                                          vertical gradient of qc, q += qc
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

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)std::max(1LL, std::min(g, 152LL * 16));
}

cudaError_t launch_qsource(const StepArgs& a, cudaStream_t st) {
  qsource_kernel<<<grid_for(std::max<long long>(a.n3, a.Ne)), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_corrector(const StepArgs& a, cudaStream_t st) {
  corrector_edges_kernel<<<grid_for(a.ncedge), 256, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  corrector_cells_kernel<<<grid_for(a.ncomp), 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace sgpu
