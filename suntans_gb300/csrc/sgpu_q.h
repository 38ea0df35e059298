// sgpu_q.h -- device argument blocks of the two solver kernels.
#pragma once
#include <cuda_runtime.h>
#include "sgpu_common.cuh"

namespace sgpu {

// Arguments of the pressure-solve kernel (all pointers are device memory).
struct QArgs {
  int F;            // maxfaces
  int ncomp;        // computational columns [0, ncomp)
  int ncols;        // all columns
  int n3c;          // storage slots of the computational columns
  int n3;           // storage slots of all columns
  int ntiles;
  int maxiters;
  double qepsilon;
  double resnorm;
  // static grid (device order)
  const int* dcoff;     // [ncols+1]
  const int* tile_col;  // [ntiles+1]
  const int* slotcol;   // [n3c] column of each computational storage slot
  const int* nk;        // [ncols]
  const int* nbr;       // [ncomp*F] neighbour column or -1
  const int* fedge;     // [ncomp*F] edge index
  const int* nke;       // [Ne]
  const int* eoff;      // [Ne+1]
  const double* Ac;     // [ncols]
  // per-solve inputs
  const int* ctop;      // [ncols]
  const double* dzz;    // [n3]
  const double* dzf;    // [sum Nke] edge order
  const double* D;      // [Ne]
  const double* q_in;   // [n3]
  const double* src_in; // [n3]
  const double* c_in;   // [n3] (read at boundary columns, qprecond 1)
  // derived per solve
  int* fmeta;           // [ncomp*F] kmin | kmax<<16, -1 = no neighbour
  int* fnoff;           // [ncomp*F] neighbour column storage offset
  double* coef;         // [n3+1]
  double* fc;           // [F*n3c]
  int* nslot;           // [F*n3c] neighbour slot of each slot and face (the slot
                        // itself where the face does not couple: fc is 0 there)
  unsigned char* sflag; // [n3c] bit 0: wet (k >= ctop); bit 1: k > ctop; bit 2: k < nk-1
  double* c;            // [n3]
  double* tw;           // [n3c] Thomas multipliers
  double* tib;          // [n3c] Thomas inverse pivots
  // working vectors [n3]
  double* x;
  double* p;
  double* r;
  double* z;
  double* rt;
  // control
  SolveCtl* ctl;
  double* partials;     // [2*grid]
};

// Arguments of the free-surface kernel.
struct HArgs {
  int F;
  int ncomp;            // computational cells [0, ncomp)
  int ncells;           // all cells
  int maxiters;
  int hprecond;
  double epsilon;
  double resnorm;
  double tmp;           // grav*(theta*dt)^2 (HCoefficients, main/phys.c:3255)
  int cpc;              // computational cells per CTA (CTA b owns [b*cpc, (b+1)*cpc))
  const int* nbr;       // [ncomp*F] neighbour cell (device order) or -1
  const int* fedge;     // [ncomp*F]
  const double* Ac;     // [ncells]
  const double* df;     // [Ne]
  const double* dg;     // [Ne]
  const double* D;      // [Ne]
  const double* h_in;   // [ncells]
  const double* b_in;   // [ncells] right-hand side (htmp)
  double* hcoef;        // [ncomp]
  double* ihcoef;       // [ncomp] 1/hcoef (the Jacobi step as a product)
  double* hf;           // [F*ncomp]
  int* hn;              // [F*ncomp] neighbour or self (coefficient 0)
  double* x;
  double* p;            // the direction, double-buffered with p1
  double* p1;
  double* r;
  double* z;
  double* rt;
  SolveCtl* ctl;
  double* partials;
};

int q_max_grid(int qprecond, int device);
cudaError_t q_launch(const QArgs& a, int qprecond, int grid, cudaStream_t st);
int h_max_grid(int device);
int h_block();  // threads per CTA of the free-surface kernel
cudaError_t h_launch(const HArgs& a, int grid, cudaStream_t st);

}  // namespace sgpu
