// sgpu_batch.h -- device data of the batched mixed-precision pressure solver.
//
// Many independent grids ("instances") share one set of device arrays: every
// instance owns a contiguous range of storage slots (one slot per cell level,
// columns z-contiguous), of columns, of edge slots and of tiles.  One
// persistent cooperative kernel advances every active instance by one CG
// iteration per global iteration; each instance keeps its own scalars,
// tolerance, iteration count and status.
#pragma once
#include <cuda_runtime.h>
#include "sgpu_common.cuh"

namespace sgpu {

constexpr int kMaxF = 8;        // faces per cell supported by the batched engine

// Instance lifecycle inside the persistent kernel.
enum InstState : int { INST_EMPTY = 0, INST_SETUP = 1, INST_RUN = 2, INST_DONE = 3 };

// Per-instance scalars and bookkeeping (device memory, one per instance slot).
struct __align__(64) BInst {
  // static description
  int t0, t1;          // tile range [t0, t1)
  int s0, s1;          // computational storage range [s0, s1) (tiles cover it)
  int maxiters;
  int qprecond;
  double tol2;         // tolerance squared
  double resnorm;
  // state
  int state;           // InstState
  int n;               // iterations executed
  int status;          // SGPU_* code
  int flags;           // bit0: reliable update now; bit1: final merge (no verification)
  int cnt;             // tiles finished in the current phase (last one reduces)
  int par;             // which p buffer holds the current direction
  int nrel;            // reliable updates done
  int s2;              // end of the instance's storage (boundary columns in [s1, s2))
  double alpha, eps, eps0, eps_ref;   // CG scalars (FP64)
  double mu, nu;
  double alpha_prev;
};

// Column metadata (one entry per computational column, global column index).
struct BCol {
  int s;               // first storage slot of the column
  int nk;              // levels stored
  int ctop;            // first wet level
  int inst;            // instance slot
};

// One face of a computational column: neighbour and the wet range shared.
struct BFace {
  int ns;              // neighbour's first storage slot, -1 = no neighbour
  int es;              // edge's first slot in edge storage (dzf-form coefficients)
  short kmin, kmax;    // levels [kmin, kmax) couple across this face
  float D;             // D of the edge (FP32 copy)
  double D64;          // D of the edge (FP64)
};

struct BatchArgs {
  int F;
  int ntiles;
  int ninst;           // instance slots in use (some may be EMPTY/DONE)
  int max_iters_chunk; // global iterations allowed in this launch
  double delta2;       // reliable-update trigger: eps < delta2 * eps_ref
  // tiles
  const int* tile_c0;    // [2*ntiles] (first, end) global column of each tile
  const int* tile_inst;  // [ntiles]
  // columns (global, computational only) and faces
  const BCol* col;       // [ncols]
  const BFace* face;     // [ncols*F]
  const double* colAc;   // [ncols]
  // per-slot FP64 inputs and derived data
  const double* dzz64;   // [nslots]
  const double* src64;   // [nslots]
  const double* q64;     // [nslots] warm start (and fixed values at boundary columns)
  const double* cin64;   // [nslots] c at boundary columns (qprecond 1)
  const double* dzfD64;  // [nedge_slots] dzf*D per edge level (qprecond 0/2)
  double* c64;           // [nslots] sqrt|diag| (qprecond 1), 1 elsewhere
  double* coef64;        // [nslots+1] vertical coefficient (scaled for qprecond 1)
  double* fc64;          // [F*nslots] face coefficients of the FP64 operator
  double* x64;           // [nslots] FP64 iterate (scaled variables for qprecond 1)
  double* b64;           // [nslots] FP64 right-hand side (scaled for qprecond 1)
  // FP32 inner data
  float* dzz32;          // [nslots]
  float* cinv32;         // [nslots] 1/c (qprecond 1)
  float* coef32;         // [nslots+1] vertical coefficient (qprecond 0/2)
  float* dzfD32;         // [nedge_slots]
  float* tw32;           // [nslots] Thomas factors (qprecond 2)
  float* tib32;          // [nslots]
  float* r32;            // [nslots]
  float* s32;            // [nslots] preconditioned residual (qprecond 2)
  float* pa32;           // [nslots] direction buffers (double-buffered)
  float* pb32;
  float* x32;            // [nslots] FP32 correction accumulated since the last reliable update
  float* z32;            // [nslots]
  // per-tile partial sums [ntiles*2] and instance table
  double* tpart;
  BInst* inst;
  SolveCtl* ctl;         // grid barrier + global flags
  int* gflags;           // [4]: 0 any reliable flag, 1 any active, 2 snapshot reliable, 3 snapshot active
};

}  // namespace sgpu
