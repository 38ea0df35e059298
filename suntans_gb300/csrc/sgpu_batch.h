// sgpu_batch.h -- device data of the batched mixed-precision pressure solver.
//
// Many independent grids ("instances") share one set of device arrays: every
// instance owns a contiguous range of storage slots (one slot per cell level,
// columns z-contiguous, every tile starting on a 4-slot = 16-byte boundary so
// that tiles can be moved with bulk copies), of columns, of edge slots and of
// tile headers.  One persistent cooperative kernel advances every active
// instance by one CG iteration per global iteration; each instance keeps its
// own scalars, tolerance, iteration count and status.
#pragma once
#include <cuda_runtime.h>
#include "sgpu_common.cuh"

namespace sgpu {

constexpr int kMaxF = 8;         // faces per cell supported by the batched engine
constexpr int kBTSlots = 1024;   // storage slots per tile (4 per thread of a 256-thread CTA)
constexpr int kBTCols = 128;     // columns per tile
constexpr int kBTFaces = 512;    // column-faces per tile (ncols * F)
constexpr int kHdrCap = 10240;   // bytes of a tile header (see tile header layout below)
constexpr int kStreamFloats = kBTSlots + 4;                 // one FP32 stream of a tile (+1 group)
constexpr int kStreamBytes = kStreamFloats * 4;             // 4112, a multiple of 16
constexpr int kBufBytes = kHdrCap + 4 * kStreamBytes;       // the smallest pipeline stage (4 streams)
// A stage holds the descriptor and header (at most kHdrCap bytes; each launch
// sizes it to its largest tile header) and `streams` = 4 + F FP32 streams (p,
// s, coef, one face-weight stream per face and x; the update phase uses 2 of
// them, and 4 as scratch for qprecond 2), or 5 + F in the one-pass form (+ z).
__host__ __device__ constexpr int stage_bytes_for(int streams) { return kHdrCap + streams * kStreamBytes; }
__host__ __device__ constexpr int stage_bytes_for(int hdr_cap, int streams) { return hdr_cap + streams * kStreamBytes; }
static_assert(kBTCols <= 256, "the header's slot-to-column map holds one byte per slot");
constexpr int kListCap = 512;    // tiles per CTA per phase
constexpr int kPwVals = 4;       // partial sums per warp slot (the one-pass form reduces four)
// dynamic shared memory of the kernel: 2 stages, 4 mbarriers (32 B), the tile list
__host__ __device__ constexpr int dyn_smem_bytes(int streams) { return 2 * stage_bytes_for(streams) + 32 + 4 * kListCap; }
__host__ __device__ constexpr int dyn_smem_bytes_for(int stage_bytes) { return 2 * stage_bytes + 32 + 4 * kListCap; }
constexpr int kDynSmem = dyn_smem_bytes(4);

// Tile header (global, built on the host when an instance is added; all
// offsets are multiples of 16 bytes):
//   [0]       int ncols, nslots, base, inst
//   o_start   unsigned short start[ncols+1]   slot offset of each column in the tile
//   o_cn      int cn[ncols]                   ctop | nk << 16
//   o_fns     int fns[ncols*F]                neighbour's first slot (-1: none)
//   o_fkk     int fkk[ncols*F]                kmin | kmax << 16 (empty when no neighbour)
//   o_cmap    unsigned char cmap[nslots]      column of each slot of the tile
__host__ __device__ __forceinline__ int pad16(int b) { return (b + 15) & ~15; }
struct HdrLayout {
  int o_start, o_cn, o_fns, o_fkk, o_cmap, bytes;
};
__host__ __device__ __forceinline__ HdrLayout hdr_layout(int ncols, int F, int nslots) {
  HdrLayout L;
  L.o_start = 16;
  L.o_cn = L.o_start + pad16(2 * (ncols + 1));
  const int sf = pad16(4 * ncols * F);
  L.o_fns = L.o_cn + pad16(4 * ncols);
  L.o_fkk = L.o_fns + sf;
  L.o_cmap = L.o_fkk + sf;  // the face weights travel as streams, not in the header
  L.bytes = L.o_cmap + pad16(nslots);
  return L;
}

// Per-launch tile descriptor.
struct TileDesc {
  int hdr;      // byte offset of the header in the header arena
  int hdr_bytes;
  int base;     // first storage slot (multiple of 4)
  int nslots;
  int inst;
  int c0, c1;   // global computational columns [c0, c1)
  int pad;
};

// Instance lifecycle inside the persistent kernel.
enum InstState : int { INST_EMPTY = 0, INST_SETUP = 1, INST_RUN = 2, INST_DONE = 3 };

// Per-instance scalars and bookkeeping (device memory, one per instance slot).
struct __align__(64) BInst {
  // static description
  int t0, t1;          // tile range [t0, t1) in this launch's tile list
  int s0, s1;          // computational storage range [s0, s1) (tiles cover it)
  int maxiters;
  int qprecond;
  double tol2;         // tolerance squared
  double resnorm;
  // state
  int state;           // InstState
  int n;               // iterations executed
  int status;          // SGPU_* code
  int flags;           // bit0: reliable update now; bit1: final merge; bit2: last chance at maxiters
  int cnt;             // tiles finished in the current phase (the last flush reduces)
  int par;             // which p buffer holds the current direction (and, in the one-pass
                       // form, which r and z buffers hold the current residual and A p)
  int nrel;            // reliable updates done
  int s2;              // end of the instance's storage (boundary columns in [s1, s2))
  int stride;          // iterates on a launch's global iterations it with it % stride == 0
                       // (0 or 1: on every one); sgpu_batch_set_stride
  double alpha, eps, eps0, eps_ref;   // CG scalars (FP64)
  double mu, nu;
  double alpha_prev;
  double nu_x;         // the solution increment nu_x * p still to add to x32 (p = the
                       // direction of the last update phase): the next apply phase
                       // adds it where it streams that direction anyway, or the
                       // reliable update adds it; 0 when nothing is pending.  The
                       // one-pass form keeps its pending step in nu instead (applied
                       // to r and x by the next pass) and leaves nu_x at 0
};

// Column metadata (one entry per computational column, global column index),
// used by the set-up and FP64 residual phases.
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
  int stage_bytes;     // bytes of one pipeline stage: hdr_cap + streams * kStreamBytes
  int hdr_cap;         // bytes before a stage's streams: descriptor + the launch's largest header
  int stream_floats;   // floats per stage stream: the launch's largest tile + 4
  int x_in_apply;      // 1: the solution update x32 += nu p runs in the next apply pass, where
                       // p is streamed anyway; 0: in the update pass (streams p and x there)
  int one_pass;        // 1 (qprecond 0/1): one pass per iteration -- r -= nu z, x += nu p,
                       // p = r + mu p and z = A p in one sweep, mu from the pass's inner
                       // products (r, z and p double-buffered); 0: the two passes above
  int ntiles;
  int ninst;           // instance slots in use (some may be EMPTY/DONE)
  int max_iters_chunk; // global iterations allowed in this launch
  double delta2;       // reliable-update trigger: eps < delta2 * eps_ref
  // tiles
  const TileDesc* tiles;       // [ntiles]
  const int* tile_inst;        // [ntiles]
  const unsigned char* hdrs;   // header arena
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
  double* c64;           // [nslots] 1/sqrt|diag| (qprecond 1: 1/c), 1 elsewhere
  double* coef64;        // [nslots+4] vertical coefficient (scaled for qprecond 1)
  double* fc64;          // [F*nslots] face coefficients of the FP64 operator (qprecond 1)
  double* x64;           // [nslots] FP64 iterate (scaled variables for qprecond 1)
  double* b64;           // [nslots] FP64 right-hand side (scaled for qprecond 1)
  // FP32 inner data
  float* fz32;           // [nslots] dzz/c (qprecond 1 face coefficients)
  float* fw32;           // [F][fw_stride] face weights, FP32: (dzz/c_u) D (1/c_n) for qprecond 1, dzf*D else
  long long fw_stride;
  float* cinv32;         // [nslots] 1/c (qprecond 1)
  float* coef32;         // [nslots+4] vertical coefficient (scaled for qprecond 1)
  float* dzfD32;         // [nedge_slots]
  float* tw32;           // [nslots] Thomas factors (qprecond 2)
  float* tib32;          // [nslots]
  float* r32;            // [nslots]
  float* s32;            // [nslots] preconditioned residual (qprecond 2)
  float* pa32;           // [nslots] direction buffers (double-buffered)
  float* pb32;
  float* x32;            // [nslots] FP32 correction accumulated since the last reliable update
  float* z32;            // [nslots]
  float* r2_32;          // [nslots] second residual buffer (one-pass form; qprecond 0/1)
  float* z2_32;          // [nslots] second A p buffer (one-pass form; qprecond 0/1)
  // per-CTA partial sums [ntiles*2] of the simple phases and instance table
  double* tpart;
  double* tpw;           // [ntiles*8*kPwVals] per-warp partial sums of the pipelined phases
  BInst* inst;
  SolveCtl* ctl;         // grid barrier
  int* gflags;           // [4]: 0 any reliable flag, 2 its snapshot, 3 any instance running
};

}  // namespace sgpu
