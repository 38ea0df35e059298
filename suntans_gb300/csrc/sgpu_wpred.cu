// sgpu_wpred.cu -- WPredictor (main/phys.c:2025-2287) on the device: the
// predictor of the vertical velocity w before the pressure solve.
//
//   wp_zero_kernel    2044-2051  first step: the Adams-Bashforth histories start at 0
//   wp_wc_kernel      2100-2103  w at cell centres (for the advective face values)
//   wp_face_kernel    4908-4948  first-order upwind face values of w on the
//                                computational edges (GetMomentumFaceValues)
//   wp_column_kernel  2071-2241  per computational column: Adams-Bashforth
//                                start, pressure gradient, advection, horizontal
//                                diffusion and wall drag (in the reference's edge
//                                order), the new history Cn_W
//   wp_solve_kernel   2246-2284  per computational column: vertical diffusion,
//                                explicit part and the tridiagonal solve for w
//
// Every expression is evaluated in the reference's order with explicitly
// rounded operations, so w, Cn_W and Cn_W2 are the reference's bits.  The
// column kernel gathers the horizontal-diffusion terms the reference scatters
// edge by edge; each column's list of its computational edges keeps the
// reference's edge order, which is the order of the additions.  Where a column
// is deeper than a face's edge the reference reads its face-value scratch past
// the edge's levels (zero memory); those terms are 0 here.
#include "sgpu_step.h"

namespace sgpu {

namespace {
__device__ __forceinline__ double ADD(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ double SUB(double x, double y) { return __dsub_rn(x, y); }
__device__ __forceinline__ double MUL(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ double DIV(double x, double y) { return __ddiv_rn(x, y); }

__device__ void thomas_rn(double* a, double* b, double* c, double* d, double* u, int N) {  // util.c:185-203
  for (int k = 1; k < N; ++k) {
    b[k] = SUB(b[k], DIV(MUL(a[k], c[k - 1]), b[k - 1]));
    d[k] = SUB(d[k], DIV(MUL(a[k], d[k - 1]), b[k - 1]));
  }
  u[N - 1] = DIV(d[N - 1], b[N - 1]);
  for (int k = N - 2; k >= 0; --k) u[k] = SUB(DIV(d[k], b[k]), DIV(MUL(c[k], u[k + 1]), b[k]));
}

int blocks(long long n, int bs) {
  long long b = (n + bs - 1) / bs;
  return (int)std::max(1LL, std::min(b, 152LL * 16));
}
}  // namespace

__global__ void wp_zero_kernel(WPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < A.n3; u += T) A.Cn_W[u] = A.Cn_W2[u] = 0;
}

__global__ void wp_wc_kernel(WPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.Nc; j += T) {
    const double* w = A.w + A.woff[j];
    double* wc = A.wc + A.dcoff[j];
    for (int k = A.ctop[j]; k < A.nk[j]; ++k) wc[k] = MUL(0.5, ADD(w[k], w[k + 1]));
  }
}

__global__ void wp_face_kernel(WPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A.ncedge; t += T) {
    const int j = A.cedge[t];
    const int c1 = A.grad[2 * j], c2 = A.grad[2 * j + 1];
    const int kmin = max(A.ctop[c1], A.ctop[c2]), nk = A.nke[j], eo = A.eoff[j];
    for (int k = 0; k < kmin && k < nk; ++k) A.ut[eo + k] = 0;
    const double* w1 = A.wc + A.dcoff[c1];
    const double* w2 = A.wc + A.dcoff[c2];
    for (int k = kmin; k < nk; ++k) A.ut[eo + k] = A.utmp2[eo + k] > 0 ? w2[k] : w1[k];
  }
}

// One pass down the column: every level's terms are summed in the
// reference's order (faces, the vertical term, then the edges in edge
// order), and the history at k needs only the sums at k-1 and k, so nothing
// is kept per level but two sums; each face's and each edge's data sit in
// registers (at most kMaxF of each).
constexpr int kMaxF = 8;
__global__ void __launch_bounds__(128) wp_column_kernel(WPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.ncomp; j += T) {
    const int ct = A.ctop[j], nk = A.nk[j], co = A.dcoff[j];
    const double* w = A.w + A.woff[j];
    const double* z = A.dzz + co;
    const double* q = A.q + co;
    const double Ac = A.Ac[j];
    const double tdt = MUL(2.0, A.dt);
    // faces (advection)
    int f_eo[kMaxF], f_top[kMaxF];
    double f_c[kMaxF];
    const int nf = A.nonlinear ? A.nfaces[j] : 0;
#pragma unroll
    for (int f = 0; f < kMaxF; ++f)
      if (f < nf) {
        const int ne = A.fedge[j * A.F + f];
        f_eo[f] = A.eoff[ne];
        f_top[f] = A.nke[ne];
        f_c[f] = A.df[ne];  // times the normal below, in the reference's order
      }
    // computational edges of the column, in the reference's edge order
    const int p0 = A.ecsr[j], ned = min(A.ecsr[j + 1] - p0, kMaxF);
    int e_kmin[kMaxF], e_ne[kMaxF], e_side[kMaxF], e_w1[kMaxF], e_w2[kMaxF], e_l1[kMaxF], e_l2[kMaxF];
    double e_df[kMaxF], e_dg[kMaxF];
#pragma unroll
    for (int p = 0; p < kMaxF; ++p)
      if (p < ned) {
        const int e = A.eside[p0 + p] >> 1;
        const int c1 = A.grad[2 * e], c2 = A.grad[2 * e + 1];
        e_side[p] = A.eside[p0 + p] & 1;
        e_kmin[p] = max(A.ctop[c1], A.ctop[c2]);
        e_ne[p] = A.nke[e];
        e_w1[p] = A.woff[c1];
        e_w2[p] = A.woff[c2];
        e_l1[p] = A.dcoff[c1];
        e_l2[p] = A.dcoff[c2];
        e_df[p] = A.df[e];
        e_dg[p] = A.dg[e];
      }
    const double aAc = MUL(1.0, Ac);
    double st_prev = 0;
    for (int k = ct; k < nk; ++k) {
      // Adams-Bashforth start and the pressure gradient (2071-2089)
      const double c1v = A.Cn_W[co + k];
      double wt = ADD(ADD(w[k], MUL(A.fab2, c1v)), MUL(A.fab3, A.Cn_W2[co + k]));
      A.Cn_W2[co + k] = c1v;
      if (k > ct)
        wt = SUB(wt, MUL(DIV(tdt, ADD(z[k - 1], z[k])), SUB(q[k - 1], q[k])));
      else
        wt = ADD(wt, MUL(DIV(tdt, z[ct]), q[ct]));
      // the level's source: advection (2118-2146), diffusion and wall drag (2159-2185)
      double st = 0;
      if (A.nonlinear) {
#pragma unroll
        for (int f = 0; f < kMaxF; ++f)
          if (f < nf && k < f_top[f]) {
            const double nrm = (double)A.normal[j * A.F + f];
            st = ADD(st, DIV(MUL(MUL(MUL(A.ut[f_eo[f] + k], A.utmp2[f_eo[f] + k]), f_c[f]), nrm), aAc));
          }
        st = ADD(st, DIV(SUB(MUL(w[k], w[k]), MUL(w[k + 1], w[k + 1])), z[k]));
      }
#pragma unroll
      for (int p = 0; p < kMaxF; ++p)
        if (p < ned) {
          if (k >= e_kmin[p] && k < e_ne[p]) {
            const double* w1 = A.w + e_w1[p];
            const double* w2 = A.w + e_w2[p];
            const double ak =
                DIV(MUL(MUL(MUL(0.5, ADD(A.nu_H, MUL(0.5, ADD(A.nu_lax[e_l1[p] + k], A.nu_lax[e_l2[p] + k])))),
                            SUB(ADD(SUB(w2[k], w1[k]), w2[k + 1]), w1[k + 1])),
                        e_df[p]),
                    e_dg[p]);
            st = e_side[p] == 0 ? SUB(st, DIV(ak, Ac)) : ADD(st, DIV(ak, Ac));
          } else if (k >= e_ne[p]) {
            const double sw = ADD(w[k], w[k + 1]);
            st = ADD(st, DIV(MUL(MUL(MUL(MUL(0.25, A.CdW), fabs(sw)), sw), e_df[p]), Ac));
          }
        }
      // the new history (2210-2220) and the right-hand side (2236-2241)
      const double cn = k > ct ? SUB(0.0, DIV(MUL(A.dt, ADD(MUL(z[k - 1], st_prev), MUL(z[k], st))), ADD(z[k - 1], z[k])))
                               : SUB(0.0, MUL(A.dt, st));
      st_prev = st;
      A.Cn_W[co + k] = cn;
      A.wtmp[co + k] = ADD(wt, MUL(A.fab1, cn));
    }
  }
}

template <int KMAX>
__global__ void __launch_bounds__(128) wp_solve_kernel(WPredArgs A) {
  const int T = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.ncomp; j += T) {
    const int ct = A.ctop[j], nk = A.nk[j], co = A.dcoff[j];
    double* w = A.w + A.woff[j];
    const double* z = A.dzz + co;
    const double* nt = A.nu_tv + co;
    const double* nl = A.nu_lax + co;
    double wt[KMAX], a[KMAX], b[KMAX], c[KMAX];
    for (int k = ct; k < nk; ++k) wt[k] = A.wtmp[co + k];
    if (nk - ct > 1) {
      for (int k = ct + 1; k < nk; ++k) {
        a[k] = DIV(DIV(MUL(2.0, ADD(ADD(A.nu, MUL(A.lax, nl[k - 1])), nt[k - 1])), z[k - 1]), ADD(z[k], z[k - 1]));
        b[k] = DIV(DIV(MUL(2.0, ADD(ADD(A.nu, MUL(A.lax, nl[k])), nt[k])), z[k]), ADD(z[k], z[k - 1]));
      }
      b[ct] = DIV(ADD(ADD(A.nu, MUL(A.lax, nl[ct])), nt[ct]), MUL(z[ct], z[ct]));
      a[ct] = b[ct];
      const double ex = MUL(A.dt, SUB(1.0, A.theta));
      for (int k = ct + 1; k < nk; ++k)
        wt[k] = ADD(wt[k], MUL(ex, ADD(SUB(MUL(a[k], w[k - 1]), MUL(ADD(a[k], b[k]), w[k])), MUL(b[k], w[k + 1]))));
      const double s = ADD(a[ct], b[ct]);
      wt[ct] = ADD(wt[ct], MUL(ex, ADD(MUL(-s, w[ct]), MUL(s, w[ct + 1]))));
      const double tp = MUL(A.dt, A.theta), td = MUL(-A.dt, A.theta);
      for (int k = ct; k < nk; ++k) {
        c[k] = ADD(1.0, MUL(tp, ADD(a[k], b[k])));
        a[k] = MUL(a[k], td);
        b[k] = MUL(b[k], td);
      }
      b[ct] = ADD(b[ct], a[ct]);
      thomas_rn(a + ct, c + ct, b + ct, wt + ct, w + ct, nk - ct);
    } else {
      for (int k = ct; k < nk; ++k) w[k] = wt[k];
    }
  }
}

template <int KMAX>
static void wp_columns(const WPredArgs& a, cudaStream_t st) {
  const int nb = blocks(a.ncomp, 128);
  wp_column_kernel<<<nb, 128, 0, st>>>(a);
  wp_solve_kernel<KMAX><<<nb, 128, 0, st>>>(a);
}

cudaError_t launch_wpredictor(const WPredArgs& a, cudaStream_t st) {
  if (a.first) wp_zero_kernel<<<blocks(a.n3, 256), 256, 0, st>>>(a);
  if (a.nonlinear) {
    wp_wc_kernel<<<blocks(a.Nc, 256), 256, 0, st>>>(a);
    if (a.ncedge > 0) wp_face_kernel<<<blocks(a.ncedge, 256), 256, 0, st>>>(a);
  }
  if (a.ncomp > 0) {
    if (a.kmax <= 16) wp_columns<16>(a, st);
    else if (a.kmax <= 32) wp_columns<32>(a, st);
    else if (a.kmax <= 64) wp_columns<64>(a, st);
    else wp_columns<128>(a, st);
  }
  return cudaGetLastError();
}

}  // namespace sgpu
