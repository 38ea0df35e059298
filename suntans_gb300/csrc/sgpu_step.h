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

cudaError_t launch_update_dz(const VGridArgs& a, cudaStream_t st);
cudaError_t launch_set_flux_height(const VGridArgs& a, cudaStream_t st);
cudaError_t launch_qsource(const StepArgs& a, cudaStream_t st);
cudaError_t launch_corrector(const StepArgs& a, cudaStream_t st);

}  // namespace sgpu
