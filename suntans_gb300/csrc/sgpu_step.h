// sgpu_step.h -- argument block of the ComputeQSource / Corrector kernels.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>

namespace sgpu {

struct StepArgs {
  int n3, n3c;          // storage slots: all columns, computational columns
  int ncomp, Ne, F;
  int ncedge;           // computational edges
  double thetafactor;   // (1 - theta) / theta
  double dt;
  // static grid, device order
  const int* dcoff;     // [Nc+1]
  const int* woff;      // [Nc+1] offsets of the Nk+1-level fields
  const int* slotcol;   // [n3c]
  const int* nk;        // [Nc]
  const int* nfaces;    // [ncomp]
  const int* fedge;     // [ncomp*F]
  const int* normal;    // [ncomp*F]
  const int* nke;       // [Ne]
  const int* eoff;      // [Ne+1]
  const int* grad;      // [2*Ne] device columns of the edge's two cells (-1 none)
  const int* cedge;     // [ncedge] computational edges
  const double* Ac;     // [Nc]
  const double* df;     // [Ne]
  const double* dg;     // [Ne]
  // per step
  const int* ctop;      // [Nc]
  const int* etop;      // [Ne]
  const double* dzz;    // [n3]
  const double* dzf;    // [ne3]
  const double* u;      // [ne3]  u* (ComputeQSource)
  const double* utmp2;  // [ne3]
  const double* w;      // [nw3]  w* (ComputeQSource)
  const double* wtmp2;  // [nw3]
  const double* qc;     // [n3]   pressure correction (Corrector)
  double* src;          // [n3]   out: ComputeQSource
  double* D;            // [Ne]   out: ComputeQSource; in: Corrector
  double* u_out;        // [ne3]  Corrector, in place
  double* w_out;        // [nw3]
  double* q_out;        // [n3]
};

// UpdateDZ (option 0) and SetFluxHeight: device order as above.
struct VGridArgs {
  int Nc, Ne, Nkmax, n3;
  int linearFS;
  double smoothbot, dzsmall;
  const int* dcoff;     // [Nc+1]
  const int* nk;        // [Nc]
  const int* nke;       // [Ne]
  const int* eoff;      // [Ne+1]
  const int* grad;      // [2*Ne] device columns (-1 none)
  const double* dz;     // [Nkmax]
  const double* dv;     // [Nc]
  const double* dzbot;  // [Nc]
  const double* h;      // [Nc]
  const double* u;      // [ne3]
  int* ctop;            // [Nc] in/out
  int* etop;            // [Ne] in/out
  int* ctopold;         // [Nc] out
  int* etopold;         // [Ne] out
  double* dzz;          // [n3] in/out
  double* dzzold;       // [n3] out
  double* dzf;          // [ne3] out (Nke levels per edge)
};

// UPredictor (main/phys.c:2579-3077): device order as above; edge rows of
// u, utmp, E, dzf in edge order.
struct UPredArgs {
  int Nc, Ne, ncomp, ncell3, F, ncedge, nb2, nbnd;
  int kmax;             // the local columns hold kmax levels (>= Nkmax + 1)
  double dt, theta, grav, nu, lax, thetaM;
  int nonlinear;
  const int* cedge;     // [ncedge] computational edges
  const int* b2edge;    // [nb2] type-2 edges (mark 2)
  const int* bedge;     // [nbnd] edges of marks 2-4
  const int* grad;      // [2*Ne] device columns
  const int* nke;
  const int* eoff;
  const int* dcoff;
  const int* woff;
  const int* ctop;      // [Nc] device order
  const int* etop;      // [Ne]
  const int* nfaces;    // [ncomp] computational columns
  const int* fedge;     // [ncomp*F]
  const int* normal;    // [ncomp*F]
  const int* bnfaces;   // [ncell3] type-3 columns (device columns ncomp..)
  const int* bfedge;    // [ncell3*F]
  const int* bnormal;   // [ncell3*F]
  const int* mark;      // [Ne]
  const double* n1;     // [Ne]
  const double* n2;
  const double* dzz;    // [n3]
  const double* dzf;    // [ne3]
  const double* dg;
  const double* df;
  const double* Ac;     // [Nc] device order
  const double* dv;     // [Nc] device order
  const double* tau_T;  // [Ne]
  const double* CdT;
  const double* CdB;
  const double* nu_tv;  // [n3]
  const double* nu_lax; // [n3]
  const double* w;      // [nw3]
  const double* u;      // [ne3] u at step n (read)
  double* h;            // [Nc] device order
  double* utmp;         // [ne3]
  double* E;            // [ne3]
  double* D;            // [Ne]
  double* htmp;         // [Nc] device order (computational columns written)
  double* u_out;        // [ne3]
  unsigned char* active;  // [Nc] device order
  int* nnan;            // [1] NaN count of utmp
};

cudaError_t launch_upred_vertical(const UPredArgs& a, cudaStream_t st);
cudaError_t launch_upred_rhs(const UPredArgs& a, cudaStream_t st);
cudaError_t launch_upred_open_fluxes(const UPredArgs& a, cudaStream_t st);
cudaError_t launch_upred_velocity(const UPredArgs& a, cudaStream_t st);
cudaError_t launch_upred_boundary(const UPredArgs& a, cudaStream_t st);

// WPredictor (main/phys.c:2025-2287): device order as above.
struct WPredArgs {
  int Nc, ncomp, F, ncedge, kmax, n3;
  int nonlinear, first;  // first: the reference's time step 1 (histories start from 0)
  double fab1, fab2, fab3, dt, theta, nu, nu_H, CdW, lax;
  const int* cedge;      // [ncedge] computational edges
  const int* grad;       // [2*Ne] device columns
  const int* nke;
  const int* eoff;
  const int* dcoff;
  const int* woff;
  const int* nk;         // [Nc] device order
  const int* ctop;       // [Nc] device order
  const int* nfaces;     // [ncomp]
  const int* fedge;      // [ncomp*F]
  const int* normal;     // [ncomp*F]
  const int* ecsr;       // [ncomp+1] offsets into eside
  const int* eside;      // 2*edge + side (0: the column is grad[0]) in the computational edges' order
  const double* dzz;
  const double* df;
  const double* dg;
  const double* Ac;      // device order
  const double* q;       // [n3]
  const double* nu_tv;   // [n3]
  const double* nu_lax;  // [n3]
  const double* utmp2;   // [ne3]
  double* w;             // [nw3] in/out
  double* Cn_W;          // [n3]
  double* Cn_W2;         // [n3]
  double* wtmp;          // [n3] scratch
  double* wc;            // [n3] scratch
  double* ut;            // [ne3] scratch
};

cudaError_t launch_wpredictor(const WPredArgs& a, cudaStream_t st);

cudaError_t launch_update_dz(const VGridArgs& a, cudaStream_t st);
cudaError_t launch_set_flux_height(const VGridArgs& a, cudaStream_t st);
cudaError_t launch_qsource(const StepArgs& a, cudaStream_t st);
cudaError_t launch_corrector(const StepArgs& a, cudaStream_t st);

}  // namespace sgpu
