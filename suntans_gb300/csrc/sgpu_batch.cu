// sgpu_batch.cu -- batched, mixed-precision pressure solver (CGSolveQ
// semantics, main/phys.c:2411-2550) for many independent grids in one
// persistent cooperative launch.
//
// Precision scheme ("reliable updates", a defect-correction form of CG):
//   * the CG iteration runs on FP32 vectors: operator apply, preconditioner
//     (Jacobi through the scaling of qprecond 1, the column tridiagonal solve of
//     qprecond 2), and the vector updates;
//   * every inner product (p.Ap, r.r, r.M^-1 r) is accumulated from exact
//     products of FP32 values with FP64-class accuracy: double-float per thread
//     (error-free transformations on the FP32 pipe), FP64 across threads;
//   * the solution is accumulated in FP64: the FP32 increments collected since
//     the last update are added into the FP64 iterate whenever the iterated
//     residual norm has fallen by delta (default 0.01) since the last update, and
//     the TRUE residual b - A x is then recomputed in FP64 with FP64
//     coefficients and replaces the FP32 residual (the Krylov direction p is
//     kept, so no convergence is lost).  Convergence is declared only on that
//     FP64 true residual: sqrt(eps/eps0) < qepsilon with the reference's own eps
//     and eps0 (main/phys.c:2470-2475, 2516-2524).
//
// The operators are the reference's: OperatorQC (3364-3409) with the
// coefficients of QCoefficients/ConditionQ (3420-3471, 3629-3687) for
// qprecond 1, OperatorQ (3486-3536) for qprecond 0 and 2, Preconditioner +
// TriSolve (3577-3619, util.c:185-203) for qprecond 2.  In the FP32 apply the
// qprecond 1 face coefficients are formed on the fly as (dzz_u/c_u) D (1/c_n),
// and the qprecond 0/2 face coefficients dzf*D are read from edge storage (each
// edge level serves both of its cells).
//
// Work: computational columns are packed into tiles (<= 1024 slots,
// <= 128 columns); every tile starts on a 16-byte boundary.  A CTA is 8
// compute warps plus 1 producer warp.  In the two phases of every CG
// iteration -- A (p_new = s + mu p_old formed on the fly for the cell and its
// neighbours, z = A p_new, p.z) and B (x += nu p, r -= nu z, preconditioner,
// r.s, r.r) -- the producer streams each tile's header and its contiguous FP32
// streams into a two-stage shared-memory ring with bulk asynchronous copies
// (cp.async.bulk + mbarrier), so the compute warps never wait on metadata
// chains.  The one-pass form (qprecond 0/1, a kernel instantiation of its
// own) does an iteration in one such sweep: the pending residual step, the
// solution update, the new direction and z = A p, with the next mu from the
// sweep's r.r, r.z and z.z.  Only when some problem asks for it run the
// reliable-update phases R1 (x64 += x32) and R2 (FP64 true residual).  Each
// phase ends at a grid barrier; per-problem reductions finish before it, in
// the CTA holding the problem's first tile (pipelined phases) or in the CTA
// that completes its last tile (set-up and residual phases).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/suntans_gb300.h"
#include "sgpu_batch.h"

namespace sgpu {

constexpr int kCompute = 256;              // compute threads (8 warps)
constexpr int kThreads = kCompute + 32;    // + 1 producer warp

// ---------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f2d(float f) { return (double)f; }

// Per-thread inner-product accumulator in double-float: the product of two
// floats is split exactly into p + e (TwoProduct with one FMA), p is added to
// the high word with an error-free TwoSum, and e plus the rounding error go to
// the low word.  The pair carries ~48 significant bits, so a thread's partial
// sum is as accurate as FP64 accumulation, while every operation stays on the
// FP32 pipe (GB300's FP64 pipe, which also performs f32->f64 conversions, runs
// at ~1/70 of the FP32 rate).  The intrinsics are never contracted or
// reassociated.  Thread partials are combined in FP64.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_zero(DF& s) { s.hi = 0.f; s.lo = 0.f; }
__device__ __forceinline__ void df_addprod(DF& s, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const float t = __fadd_rn(s.hi, p);
  const float bp = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s.hi = t;
  s.lo = __fadd_rn(s.lo, __fadd_rn(err, e));
}
__device__ __forceinline__ double df_value(const DF& s) { return (double)s.hi + (double)s.lo; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void csync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }  // compute warps only

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after limit_ns and reports false (the caller records
// SGPU_TIMEOUT and carries on to the next grid barrier, which ends the kernel).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity))
    if ((long long)(globaltimer_ns() - t0) > limit_ns) return false;
  return true;
}
// 1-D bulk copy global -> shared, completion counted on `bar`; 16-byte
// aligned addresses and a size that is a multiple of 16 (asserted by layout).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// FP64 sum over the 256 compute threads, fixed order; every compute thread gets it.
template <int NV>
__device__ __forceinline__ void csum(double (&v)[NV], double* s_red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = v[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) s_red[j * 8 + wid] = s;
  }
  csync();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) s += s_red[j * 8 + w];
    v[j] = s;
  }
  csync();
}

__device__ __forceinline__ int inst_state(const BatchArgs& a, int i) { return ld_volatile_int(&a.inst[i].state); }
__device__ __forceinline__ int inst_flags(const BatchArgs& a, int i) { return ld_volatile_int(&a.inst[i].flags); }

// ---------------------------------------------------------------------------
// per-instance reduction (two levels, deterministic, composition independent)
//
// A CTA accumulates its partial over all of its tiles of one instance (they
// are consecutive in its tile list) and then flushes it to slot t0 + l with
// l = (b - t0) mod G, the local index of the CTA's first tile of that instance:
// the slots used are exactly [t0, t0 + min(G, ntiles)) and their contents do not
// depend on where the instance sits in the launch's tile list.  The flush that
// completes the instance's tile count sums those slots in order and runs
// fin(I, tot) on thread 0.  Compute warps only.
// ---------------------------------------------------------------------------
template <int NV, class Fin>
__device__ __forceinline__ void flush(const BatchArgs& a, int i, int ntiles_done, double (&acc)[NV], double* s_red,
                                      int* s_flag, Fin&& fin) {
  csum<NV>(acc, s_red);
  BInst* I = a.inst + i;
  const int G = gridDim.x;
  if (threadIdx.x == 0) {
    const int t0 = I->t0, n = I->t1 - I->t0;
    const int l = ((int)blockIdx.x - t0 % G + G) % G;
#pragma unroll
    for (int v = 0; v < NV; ++v) a.tpart[2 * (t0 + l) + v] = acc[v];
    __threadfence();
    const int old = atomicAdd(&I->cnt, ntiles_done);
    *s_flag = (old + ntiles_done == n);
  }
  csync();
  if (*s_flag) {
    __threadfence();
    const int t0 = I->t0, n = I->t1 - I->t0;
    const int m = n < G ? n : G;
    double v[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int l = threadIdx.x; l < m; l += kCompute) s += ((volatile double*)a.tpart)[2 * (t0 + l) + j];
      v[j] = s;
    }
    csum<NV>(v, s_red);
    if (threadIdx.x == 0) {
      fin(I, v);
      I->cnt = 0;
      __threadfence();
    }
  }
  csync();
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
}

// ---------------------------------------------------------------------------
// simple (non-pipelined) tile access for the rare phases: set-up and the FP64
// true residual.  Metadata from BCol/BFace staged into shared memory.
// ---------------------------------------------------------------------------
struct TileSmem {
  int start[kBTCols + 1];
  int ctop[kBTCols];
  int nk[kBTCols];
  int fns[kBTFaces];
  int fkk[kBTFaces];
  int fes[kBTFaces];
  int ncols;
};
static_assert(sizeof(TileSmem) <= kBufBytes, "simple-path metadata must fit a pipeline stage");

struct TileInfo {
  int c0, c1, base, end;
};

__device__ __forceinline__ void load_tile(const BatchArgs& a, int t, TileInfo& ti, TileSmem& sm) {
  const TileDesc d = a.tiles[t];
  ti.c0 = d.c0;
  ti.c1 = d.c1;
  ti.base = d.base;
  ti.end = d.base + d.nslots;
  const int ncols = ti.c1 - ti.c0, F = a.F;
  for (int c = threadIdx.x; c < ncols; c += kCompute) {
    const BCol cc = a.col[ti.c0 + c];
    sm.start[c] = cc.s - ti.base;
    sm.ctop[c] = cc.ctop;
    sm.nk[c] = cc.nk;
  }
  for (int e = threadIdx.x; e < ncols * F; e += kCompute) {
    const BFace fc = a.face[(size_t)ti.c0 * F + e];
    sm.fns[e] = fc.ns;
    sm.fkk[e] = fc.ns < 0 ? 0 : ((int)fc.kmin | ((int)fc.kmax << 16));
    sm.fes[e] = fc.es;
  }
  if (threadIdx.x == 0) {
    sm.start[ncols] = d.nslots;
    sm.ncols = ncols;
  }
  csync();
}

__device__ __forceinline__ int col_of(const int* start, int ncols, int s) {
  int lo = 0, hi = ncols - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= s) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Walks the CTA's tiles b, b+G, ... of instances for which want(i) holds
// (compute warps), calling body(t, i, acc) per tile and flushing per instance.
template <int NV, class Want, class Body, class Fin>
__device__ __forceinline__ void for_tiles_reduce(const BatchArgs& a, double* s_red, int* s_flag, Want&& want,
                                                 Body&& body, Fin&& fin) {
  const int G = gridDim.x;
  int cur = -1, cnt = 0;
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
  for (int t = blockIdx.x; t < a.ntiles; t += G) {
    const int i = a.tile_inst[t];
    // uniform across the CTA: an instance's state/flags change only in its
    // finaliser, which runs after every CTA has flushed all its tiles of it
    if (!want(i)) continue;
    if (i != cur) {
      if (cur >= 0) flush<NV>(a, cur, cnt, acc, s_red, s_flag, fin);
      cur = i;
      cnt = 0;
    }
    body(t, i, acc);
    ++cnt;
  }
  if (cur >= 0) flush<NV>(a, cur, cnt, acc, s_red, s_flag, fin);
}

template <class Want, class Body>
__device__ __forceinline__ void for_tiles(const BatchArgs& a, Want&& want, Body&& body) {
  for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
    const int i = a.tile_inst[t];
    if (want(i)) body(t, i);
  }
}

// ---- FP64 operator (true residual), one active slot ----
template <int QP>
__device__ __forceinline__ double apply64(const BatchArgs& a, const TileSmem& sm, int c, int u, int k, int ctop,
                                          int nk, const double* x) {
  const int F = a.F;
  double y;
  if (QP == 1) {
    y = -x[u];
    for (int f = 0; f < F; ++f) {
      const int kk = sm.fkk[c * F + f];
      if (k < (kk & 0xffff) || k >= (kk >> 16)) continue;
      y += x[sm.fns[c * F + f] + k] * a.fc64[(size_t)F * u + f];
    }
    if (k > ctop) y += a.coef64[u] * x[u - 1];
    if (k < nk - 1) y += a.coef64[u + 1] * x[u + 1];
  } else {
    const double xu = x[u];
    y = 0.0;
    for (int f = 0; f < F; ++f) {
      const int kk = sm.fkk[c * F + f];
      if (k < (kk & 0xffff) || k >= (kk >> 16)) continue;
      y += (x[sm.fns[c * F + f] + k] - xu) * a.dzfD64[sm.fes[c * F + f] + k];
    }
    if (ctop < nk - 1) {
      if (k == ctop) {
        const double c0 = a.coef64[u], c1 = a.coef64[u + 1];
        y += (-2 * c0 - c1) * xu + c1 * x[u + 1];
      } else if (k == nk - 1) {
        const double c0 = a.coef64[u];
        y += c0 * x[u - 1] - c0 * xu;
      } else {
        const double c0 = a.coef64[u], c1 = a.coef64[u + 1];
        y += c0 * x[u - 1] - (c0 + c1) * xu + c1 * x[u + 1];
      }
    } else {
      y -= 2.0 * a.coef64[u] * xu;
    }
  }
  return y;
}

// FP32 Thomas solve of one column with FP32 factors (qprecond 2); r read from
// `rin` indexed from `rbase` (global arrays: rbase 0; a staged tile: its base).
__device__ __forceinline__ void column_solve32(const BatchArgs& a, const float* rin, int rbase, int off, int ctop,
                                               int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) {
    a.s32[b] = -0.5f * rin[b - rbase] / a.coef32[b];
    return;
  }
  float dprev = rin[b - rbase];
  a.s32[b] = dprev;
  for (int u = b + 1; u < e; ++u) {
    dprev = __fmaf_rn(-a.tw32[u], dprev, rin[u - rbase]);
    a.s32[u] = dprev;
  }
  float un = a.s32[e - 1] * a.tib32[e - 1];
  a.s32[e - 1] = un;
  for (int u = e - 2; u >= b; --u) {
    un = __fmaf_rn(-a.coef32[u + 1], un, a.s32[u]) * a.tib32[u];
    a.s32[u] = un;
  }
}

// FP64 factorisation of one column (TriSolve's forward sweep), stored in FP32.
__device__ __forceinline__ void column_factor64(const BatchArgs& a, int off, int ctop, int nk) {
  const int b = off + ctop, e = off + nk;
  if (ctop == nk - 1) return;
  double bp = -2 * a.coef64[b] - a.coef64[b + 1];
  a.tib32[b] = (float)(1.0 / bp);
  for (int u = b + 1; u < e; ++u) {
    const double ak = a.coef64[u];
    const double bk = (u == e - 1) ? -a.coef64[u] : (-a.coef64[u] - a.coef64[u + 1]);
    const double bnew = bk - ak * ak / bp;
    a.tw32[u] = (float)(ak / bp);
    bp = bnew;
    a.tib32[u] = (float)(1.0 / bp);
  }
}

// ---------------------------------------------------------------------------
// per-warp partial-sum slots of the pipelined phases
//
// Slot (t0 + l, w) holds warp w's partial of CTA l of an instance whose tiles
// start at t0 (l = (b - t0) mod G as for the set-up reductions).  An empty
// slot holds kEmptyPartial, a NaN bit pattern that no arithmetic produces (a
// computed NaN is the canonical one), so the value itself signals arrival.
// ---------------------------------------------------------------------------
constexpr long long kEmptyPartial = 0x7ff4deadbeef0001LL;

__device__ __forceinline__ void st_partial(double* p, double v) {
  *(volatile long long*)p = __double_as_longlong(v);
}

// Waits (bounded) until the slot is written, returns its value and empties it.
__device__ __forceinline__ bool take_partial(double* p, long long lim, double& out) {
  volatile long long* q = (volatile long long*)p;
  long long bits = *q;
  if (bits == kEmptyPartial) {
    const unsigned long long t0 = globaltimer_ns();
    unsigned spins = 0;
    while ((bits = *q) == kEmptyPartial) {
      if (++spins > 16) __nanosleep(64);
      if ((spins & 63u) == 0 && (long long)(globaltimer_ns() - t0) > lim) {
        out = 0.0;
        return false;
      }
    }
  }
  *q = kEmptyPartial;
  out = __longlong_as_double(bits);
  return true;
}

// ---------------------------------------------------------------------------
// the pipelined phases
// ---------------------------------------------------------------------------
// One pipeline stage in shared memory: a 32-byte descriptor written by the
// producer, the tile header (room for the launch's largest header), and the
// FP32 streams.
// The descriptor carries what the compute warps need of the tile's instance
// (its scalars and its partial-sum slot), so that they never wait on a global
// load when the instance changes.
struct StageDesc {
  int base, nslots, inst, par;
  int slot;      // partial-sum slot of this CTA for the instance: t0 + ((b - t0) mod G)
  int owner;     // 1: this CTA holds the instance's first tile and finalises it
  float mu, nu;  // the instance's scalars for this phase (FP32)
};
static_assert(sizeof(StageDesc) == 32, "stage descriptor is 32 bytes");
constexpr int kStageHdrOff = 32;
__device__ __forceinline__ StageDesc* stage_desc(unsigned char* stage) { return (StageDesc*)(stage); }
__device__ __forceinline__ unsigned char* stage_hdr(unsigned char* stage) { return stage + kStageHdrOff; }
__device__ __forceinline__ float* stage_stream(unsigned char* stage, int hcap, int sfl, int k) {
  return (float*)(stage + hcap + k * 4 * sfl);
}

struct Pipe {
  unsigned char* stage[2];
  int hcap;          // bytes before the streams of a stage (BatchArgs::hdr_cap)
  int sfl;           // floats per stream (BatchArgs::stream_floats)
  uint64_t* full;    // [2]
  uint64_t* empty;   // [2]
  int* list;         // tiles of this CTA for the current phase
  int* own;          // instances this CTA finalises in the current phase
  int* nown;
  int* count;
  uint32_t seq;      // tiles consumed (compute warps) or filled (producer) so far, all phases
};

// Builds the CTA's ordered list of tiles t = b, b+G, ... with want(inst(t)).
// All 288 threads take part (it ends with __syncthreads).
template <class Want>
__device__ __forceinline__ void build_list(const BatchArgs& a, Pipe& P, Want&& want, int* s_wsum) {
  const int G = gridDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) *P.count = 0;
  __syncthreads();
  const int per = (a.ntiles - (int)blockIdx.x + G - 1) / G;  // candidate tiles of this CTA
  for (int j0 = 0; j0 < per; j0 += kCompute) {
    bool ok = false;
    int t = 0;
    if (warp < 8) {
      const int j = j0 + (int)threadIdx.x;
      t = (int)blockIdx.x + j * G;
      ok = (j < per) && want(a.tile_inst[t]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (lane == 0 && warp < 8) s_wsum[warp] = __popc(m);
    __syncthreads();
    if (ok) {
      int off = *P.count;
      for (int w = 0; w < warp; ++w) off += s_wsum[w];
      off += __popc(m & ((1u << lane) - 1u));
      if (off < kListCap) P.list[off] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < 8; ++w) tot += s_wsum[w];
      *P.count += tot;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && *P.count > kListCap) *P.count = kListCap;  // the host guarantees this never binds
  __syncthreads();
}

// Instance fields the producer hands to the compute warps with each tile.
struct ProdInst {
  int inst, par, slot, owner;
  float mu, nu, nux;
};
__device__ __forceinline__ ProdInst prod_inst(const BatchArgs& a, int i) {
  const BInst& I = a.inst[i];
  ProdInst r;
  r.inst = i;
  r.par = ld_volatile_int(&I.par);
  const int G = gridDim.x, t0 = ld_volatile_int(&I.t0);
  const int l = ((int)blockIdx.x - t0 % G + G) % G;
  r.slot = t0 + l;
  r.owner = (l == 0);
  r.mu = (float)(*(volatile const double*)&I.mu);
  r.nu = (float)(*(volatile const double*)&I.nu);
  r.nux = (float)(*(volatile const double*)&I.nu_x);
  return r;
}

// Residual and A p buffers: the one-pass form alternates between two of each
// (a pass reads the neighbours' old values while it writes its own new ones);
// the two-pass form updates r in place and writes z in the apply pass only.
__device__ __forceinline__ float* rbuf(const BatchArgs& a, int par) { return (a.one_pass && par) ? a.r2_32 : a.r32; }
__device__ __forceinline__ float* zbuf(const BatchArgs& a, int par) { return (a.one_pass && par) ? a.z2_32 : a.z32; }

// Producer: fill stage seq&1 with tile descriptor d of instance fields pi.
// PH 0 = apply, 1 = update, 2 = the one-pass form's single sweep (streams p,
// r, coef, the F face weights, z and x of the current buffers).
template <int QP, int PH>
__device__ __forceinline__ void produce(const BatchArgs& a, Pipe& P, const TileDesc& d, const ProdInst& pi,
                                        long long lim, int* err) {
  const uint32_t q = P.seq;
  const int b = q & 1;
  if (q >= 2 && !mbar_wait(&P.empty[b], ((q >> 1) - 1) & 1, lim)) *err = 1;
  const int par = pi.par;
  const int n4 = (d.nslots + 3) & ~3;
  unsigned char* st = b ? P.stage[1] : P.stage[0];
  StageDesc* sd = stage_desc(st);
  sd->base = d.base;
  sd->nslots = d.nslots;
  sd->inst = d.inst;
  sd->par = par;
  sd->slot = pi.slot;
  sd->owner = pi.owner;
  sd->mu = pi.mu;
  const bool xa = a.x_in_apply != 0;
  sd->nu = PH == 0 ? (xa ? pi.nux : 0.f) : pi.nu;  // apply: the pending solution increment's nu
  const bool hdr = (PH != 1) || (QP == 2);
  uint32_t bytes = 0;
  if (PH == 0) bytes = d.hdr_bytes + 2 * 4 * n4 + 4 * (n4 + 4) + a.F * 4 * n4 + (xa ? 4 * n4 : 0);
  else if (PH == 2) bytes = d.hdr_bytes + 4 * 4 * n4 + 4 * (n4 + 4) + a.F * 4 * n4;
  else bytes = (hdr ? d.hdr_bytes : 0) + (xa ? 2 : 4) * 4 * n4;
  fence_proxy_async();
  mbar_arrive_expect_tx(&P.full[b], bytes);
  if (hdr) bulk_g2s(stage_hdr(st), a.hdrs + d.hdr, d.hdr_bytes, &P.full[b]);
  if (PH == 2) {
    const float* pold = par ? a.pb32 : a.pa32;
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 0), pold + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 1), rbuf(a, par) + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 2), a.coef32 + d.base, 4 * (n4 + 4), &P.full[b]);
    for (int f = 0; f < a.F; ++f)
      bulk_g2s(stage_stream(st, P.hcap, P.sfl, 3 + f), a.fw32 + (size_t)f * a.fw_stride + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 3 + a.F), zbuf(a, par) + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 4 + a.F), a.x32 + d.base, 4 * n4, &P.full[b]);
  } else if (PH == 0) {
    const float* pold = par ? a.pb32 : a.pa32;
    const float* S = (QP == 2) ? a.s32 : a.r32;
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 0), pold + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 1), S + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 2), a.coef32 + d.base, 4 * (n4 + 4), &P.full[b]);
    for (int f = 0; f < a.F; ++f)
      bulk_g2s(stage_stream(st, P.hcap, P.sfl, 3 + f), a.fw32 + (size_t)f * a.fw_stride + d.base, 4 * n4, &P.full[b]);
    if (xa) bulk_g2s(stage_stream(st, P.hcap, P.sfl, 3 + a.F), a.x32 + d.base, 4 * n4, &P.full[b]);
  } else {
    if (!xa) {
      const float* p = par ? a.pb32 : a.pa32;  // the direction written by phase A
      bulk_g2s(stage_stream(st, P.hcap, P.sfl, 0), p + d.base, 4 * n4, &P.full[b]);
      bulk_g2s(stage_stream(st, P.hcap, P.sfl, 1), a.x32 + d.base, 4 * n4, &P.full[b]);
    }
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 2), a.z32 + d.base, 4 * n4, &P.full[b]);
    bulk_g2s(stage_stream(st, P.hcap, P.sfl, 3), a.r32 + d.base, 4 * n4, &P.full[b]);
  }
  P.seq = q + 1;
}

// The direction of a slot, formed where it is used.  Two-pass form: p_new =
// S + mu p_old (S = r, or s for qprecond 2).  One-pass form (M): the pending
// residual step first, r_new = r - nu z, then p_new = r_new + mu p_old.  A slot
// and each of its neighbours evaluate the same two roundings on the same
// operands, so every reader sees the value the slot's owner stores.
template <bool M>
__device__ __forceinline__ float res_new(float nu, float r, float z) {
  return M ? __fmaf_rn(-nu, z, r) : r;
}

// FP32 apply of one active slot from a staged tile (own data in shared
// memory, neighbours from global).  p_new formed on the fly (res_new above);
// M: sz / zold are the staged / global z and ru_out receives r_new of the slot.
template <int QP, bool M>
__device__ __forceinline__ float apply32(const BatchArgs& a, const unsigned char* hd, const HdrLayout& L, int c,
                                         int s, int k, int ctop, int nk, float mu, float nu, const float* sp,
                                         const float* sS, const float* sz, const float* sc, const float* sf,
                                         const float* __restrict__ pold, const float* __restrict__ S,
                                         const float* __restrict__ zold, float& pu_out, float& ru_out) {
  const int F = a.F;
  const int* fns = (const int*)(hd + L.o_fns);
  const int* fkk = (const int*)(hd + L.o_fkk);
  auto own = [&](int t) { return __fmaf_rn(mu, sp[t], res_new<M>(nu, sS[t], M ? sz[t] : 0.f)); };
  auto nbr = [&](int n) { return __fmaf_rn(mu, pold[n], res_new<M>(nu, S[n], M ? zold[n] : 0.f)); };
  ru_out = res_new<M>(nu, sS[s], M ? sz[s] : 0.f);
  const float pu = __fmaf_rn(mu, sp[s], ru_out);
  pu_out = pu;
  float y;
  if (QP == 1) {
    y = -pu;
    for (int f = 0; f < F; ++f) {
      const int kk = fkk[c * F + f];
      if (k < (kk & 0xffff) || k >= (kk >> 16)) continue;
      const int n = fns[c * F + f] + k;
      y = __fmaf_rn(sf[f * a.stream_floats + s], nbr(n), y);  // staged face weight stream f
    }
    if (k > ctop) y = __fmaf_rn(sc[s], own(s - 1), y);
    if (k < nk - 1) y = __fmaf_rn(sc[s + 1], own(s + 1), y);
  } else {
    y = 0.f;
    for (int f = 0; f < F; ++f) {
      const int kk = fkk[c * F + f];
      if (k < (kk & 0xffff) || k >= (kk >> 16)) continue;
      const int n = fns[c * F + f] + k;
      y = __fmaf_rn(nbr(n) - pu, sf[f * a.stream_floats + s], y);  // staged dzf*D of the edge level
    }
    const float c0 = sc[s];
    if (ctop < nk - 1) {
      if (k == ctop) {
        const float c1 = sc[s + 1];
        const float pp = own(s + 1);
        y += (-2.f * c0 - c1) * pu + c1 * pp;
      } else if (k == nk - 1) {
        const float pm = own(s - 1);
        y += c0 * pm - c0 * pu;
      } else {
        const float c1 = sc[s + 1];
        const float pm = own(s - 1);
        const float pp = own(s + 1);
        y += c0 * pm - (c0 + c1) * pu + c1 * pp;
      }
    } else {
      y -= 2.f * c0 * pu;
    }
  }
  return y;
}

__device__ __forceinline__ int hcol_of(const unsigned short* start, int ncols, int s) {
  int lo = 0, hi = ncols - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int)start[mid] <= s) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Branch-free FP32 apply of a thread's 4 slots of a staged tile with a
// compile-time face count: every neighbour gather of the 4 slots is
// independent of the others, so all of them are in flight together.  A face
// that does not couple a level gathers the slot itself (a valid address) with
// a zero weight.  M: the one-pass formation (res_new), rv receives r_new.
template <int QP, int FF, bool M, class Emit>
__device__ __forceinline__ void apply_tile32(const BatchArgs& a, const unsigned char* hd, const HdrLayout& L,
                                             int ncols, int len, int base, float mu, float nu, const float* sp,
                                             const float* sS, const float* sz, const float* sc, const float* sf,
                                             const float* __restrict__ pold, const float* __restrict__ S,
                                             const float* __restrict__ zold, float (&yv)[kBTSlots / kCompute],
                                             float (&pv)[kBTSlots / kCompute], bool (&on)[kBTSlots / kCompute],
                                             Emit&& emit) {
  constexpr int Q = kBTSlots / kCompute;
  const unsigned short* start = (const unsigned short*)(hd + L.o_start);
  const int* cn = (const int*)(hd + L.o_cn);
  const int* fns = (const int*)(hd + L.o_fns);
  const int* fkk = (const int*)(hd + L.o_fkk);
  const unsigned char* cmap = hd + L.o_cmap;
  auto own = [&](int t) { return __fmaf_rn(mu, sp[t], res_new<M>(nu, sS[t], M ? sz[t] : 0.f)); };
  int cc[Q], kv[Q], ctop[Q], nk[Q], sv[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int s0 = threadIdx.x + q * kCompute;
    const bool in = s0 < len;
    const int s = in ? s0 : 0;
    sv[q] = s;
    cc[q] = cmap[s];
    kv[q] = s - start[cc[q]];
    const int w = cn[cc[q]];
    ctop[q] = w & 0xffff;
    nk[q] = w >> 16;
    on[q] = in && kv[q] >= ctop[q];
  }
  // gathers, then the slots' applies; the one-pass form (three gathers per
  // face instead of two) takes the slots in two halves to stay in registers
  constexpr int NG = M ? 2 : 1, QG = Q / NG;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
  float pn[QG][FF], wn[QG][FF];
#pragma unroll
  for (int qi = 0; qi < QG; ++qi) {
    const int q = g * QG + qi;
#pragma unroll
    for (int f = 0; f < FF; ++f) {
      const int e = cc[q] * FF + f;
      const int kk = fkk[e];
      const bool ok = on[q] && kv[q] >= (kk & 0xffff) && kv[q] < (kk >> 16);
      const int n = ok ? fns[e] + kv[q] : base + sv[q];
      pn[qi][f] = __fmaf_rn(mu, pold[n], res_new<M>(nu, S[n], M ? zold[n] : 0.f));
      // staged face weight: (dzz/c_u) D (1/c_n) for qprecond 1, dzf*D of the
      // edge level otherwise (0 where the face does not couple)
      wn[qi][f] = sf[f * a.stream_floats + sv[q]];
    }
  }
#pragma unroll
  for (int qi = 0; qi < QG; ++qi) {
    const int q = g * QG + qi;
    const int s = sv[q], k = kv[q];
    const float ru = res_new<M>(nu, sS[s], M ? sz[s] : 0.f);
    const float pu = __fmaf_rn(mu, sp[s], ru);
    float y;
    if (QP == 1) {
      y = -pu;
#pragma unroll
      for (int f = 0; f < FF; ++f) y = __fmaf_rn(wn[qi][f], pn[qi][f], y);
      if (k > ctop[q]) y = __fmaf_rn(sc[s], own(s - 1), y);
      if (k < nk[q] - 1) y = __fmaf_rn(sc[s + 1], own(s + 1), y);
    } else {
      y = 0.f;
#pragma unroll
      for (int f = 0; f < FF; ++f) y = __fmaf_rn(pn[qi][f] - pu, wn[qi][f], y);
      const float c0 = sc[s];
      if (ctop[q] < nk[q] - 1) {
        if (k == ctop[q]) {
          const float c1 = sc[s + 1];
          const float pp = own(s + 1);
          y += (-2.f * c0 - c1) * pu + c1 * pp;
        } else if (k == nk[q] - 1) {
          const float pm = own(s - 1);
          y += c0 * pm - c0 * pu;
        } else {
          const float c1 = sc[s + 1];
          const float pm = own(s - 1);
          const float pp = own(s + 1);
          y += c0 * pm - (c0 + c1) * pu + c1 * pp;
        }
      } else {
        y -= 2.f * c0 * pu;
      }
    }
    if (M) {
      emit(q, on[q], y, pu, ru);
    } else {
      yv[q] = on[q] ? y : 0.f;
      pv[q] = pu;
    }
  }
  }
}

// One pipelined phase over the CTA's list.  PH 0: apply; PH 1: update.
template <int QP, int PH, class Fin>
__device__ __forceinline__ void pipelined_phase(const BatchArgs& a, Pipe& P, double* s_red, int* s_flag,
                                                long long lim, Fin&& fin) {
  const int n = *P.count;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int err = 0;
  if (warp == 8) {
    // producer warp: lane 0 issues every fill of this phase in list order.
    // Tile descriptors are loaded one tile ahead; the instance fields are
    // re-read only when the instance changes.
    if (lane == 0 && n > 0) {
      TileDesc dn = a.tiles[P.list[0]];
      ProdInst pi;
      pi.inst = -1;
      for (int j = 0; j < n; ++j) {
        const TileDesc d = dn;
        if (j + 1 < n) dn = a.tiles[P.list[j + 1]];
        if (d.inst != pi.inst) pi = prod_inst(a, d.inst);
        produce<QP, PH>(a, P, d, pi, lim, &err);
      }
    }
    P.seq = __shfl_sync(0xffffffffu, P.seq, 0);
    err = __shfl_sync(0xffffffffu, err, 0);
    if (lane == 0 && err) atomicCAS(&a.ctl->status, SGPU_OK, SGPU_TIMEOUT);
    return;
  }
  // sums per phase: apply p.z; update r.r (qprecond 2: r.s, r.r); one pass
  // p.z, r.r, r.z, z.z
  constexpr int NV = PH == 2 ? 4 : ((PH == 1 && QP == 2) ? 2 : 1);
  static_assert(NV <= kPwVals, "warp slots hold kPwVals sums");
  // The accumulators are scalars, not arrays: an array captured by reference
  // in the flush lambda below would live in local memory, and every
  // accumulation of the phase loops would load and store it there.
  DF dacc0, dacc1, dacc2, dacc3;
  df_zero(dacc0);
  df_zero(dacc1);
  df_zero(dacc2);
  df_zero(dacc3);
  // Per-warp flush of the instance's partial sums: a fixed shuffle tree, then
  // lane 0 stores the warp's value into the CTA's slot.  No barrier, fence or
  // atomic: the owner CTA collects the slots at the end of the phase.
  // `enc` is the slot, bitwise complemented when this CTA owns the instance.
  if (threadIdx.x == 0) *P.nown = 0;
  auto do_flush = [&](int inst, int enc) {
    double v0 = df_value(dacc0), v1 = df_value(dacc1), v2 = df_value(dacc2), v3 = df_value(dacc3);
    df_zero(dacc0);
    df_zero(dacc1);
    df_zero(dacc2);
    df_zero(dacc3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v0 += __shfl_xor_sync(0xffffffffu, v0, o);
      if (NV >= 2) v1 += __shfl_xor_sync(0xffffffffu, v1, o);
      if (NV == 4) {
        v2 += __shfl_xor_sync(0xffffffffu, v2, o);
        v3 += __shfl_xor_sync(0xffffffffu, v3, o);
      }
    }
    const int slot = enc < 0 ? ~enc : enc;
    if (lane == 0) {
      double* w = a.tpw + ((size_t)slot * 8 + warp) * kPwVals;
      st_partial(w, v0);
      if (NV >= 2) st_partial(w + 1, v1);
      if (NV == 4) {
        st_partial(w + 2, v2);
        st_partial(w + 3, v3);
      }
    }
    if (enc < 0 && threadIdx.x == 0) P.own[(*P.nown)++] = inst;
  };
  int cur = -1, cur_enc = 0;
  for (int j = 0; j < n; ++j) {
    const uint32_t q = P.seq;
    const int b = q & 1;
    if (!mbar_wait(&P.full[b], (q >> 1) & 1, lim)) err = 1;
    unsigned char* st = b ? P.stage[1] : P.stage[0];
    const StageDesc sd = *stage_desc(st);
    if (sd.inst != cur) {
      if (cur >= 0) do_flush(cur, cur_enc);
      cur = sd.inst;
      cur_enc = sd.owner ? ~sd.slot : sd.slot;
    }
    const float mu = sd.mu, nu = sd.nu;
    const int len = sd.nslots;
    const int base = sd.base;
    constexpr int Q = kBTSlots / kCompute;
    if (PH == 0 || PH == 2) {
      constexpr bool M = PH == 2;
      const unsigned char* hd = stage_hdr(st);
      const int ncols = ((const int*)hd)[0];
      const HdrLayout L = hdr_layout(ncols, a.F, len);
      const unsigned short* start = (const unsigned short*)(hd + L.o_start);
      const int* cn = (const int*)(hd + L.o_cn);
      const float* sp = stage_stream(st, P.hcap, P.sfl, 0);
      const float* sS = stage_stream(st, P.hcap, P.sfl, 1);
      const float* sc = stage_stream(st, P.hcap, P.sfl, 2);
      const float* sf = stage_stream(st, P.hcap, P.sfl, 3);
      const float* sz = M ? stage_stream(st, P.hcap, P.sfl, 3 + a.F) : nullptr;
      const float* pold = sd.par ? a.pb32 : a.pa32;
      float* pnew = sd.par ? a.pa32 : a.pb32;
      const float* S = M ? rbuf(a, sd.par) : ((QP == 2) ? a.s32 : a.r32);
      const float* zold = M ? zbuf(a, sd.par) : nullptr;
      float* rnew = M ? rbuf(a, sd.par ^ 1) : nullptr;
      float* znew = M ? zbuf(a, sd.par ^ 1) : a.z32;
      // the pending solution increment x32 += nu p_old, applied here where its
      // direction is staged anyway: 4 consecutive slots per thread (padding
      // slots hold zeros in every stream).  Two-pass form: nu is the previous
      // update phase's step; one pass: the step this pass also applies to r.
      const float mu_p = mu, nu_r = M ? nu : 0.f;
      {
        const int s0 = 4 * (int)threadIdx.x;
        if (nu != 0.f && s0 < len) {
          const float* sx = stage_stream(st, P.hcap, P.sfl, M ? 4 + a.F : 3 + a.F);
          const float4 p4 = *(const float4*)(sp + s0);
          const float4 x4 = *(const float4*)(sx + s0);
          *(float4*)(a.x32 + base + s0) = make_float4(__fmaf_rn(nu, p4.x, x4.x), __fmaf_rn(nu, p4.y, x4.y),
                                                      __fmaf_rn(nu, p4.z, x4.z), __fmaf_rn(nu, p4.w, x4.w));
        }
      }
      // Two-pass apply: z and p_new are stored after the stage is handed back.
      // One pass: each slot's r_new, p_new and z are stored and summed as soon
      // as they are formed (four slots' worth of them would not fit in
      // registers beside the gathers).
      float yv[Q], pv[Q];
      bool on[Q];
      // (captures scalars only: an array captured here would live in local memory)
      const int ubase = base + (int)threadIdx.x;
      auto emit = [&](int qq, bool o, float y, float pu, float ru) {
        if (!o) return;
        const int u = ubase + qq * kCompute;
        znew[u] = y;
        pnew[u] = pu;
        rnew[u] = ru;
        df_addprod(dacc0, pu, y);
        df_addprod(dacc1, ru, ru);
        df_addprod(dacc2, ru, y);
        df_addprod(dacc3, y, y);
      };
      if (a.F == 3) {
        apply_tile32<QP, 3, M>(a, hd, L, ncols, len, base, mu_p, nu_r, sp, sS, sz, sc, sf, pold, S, zold, yv, pv, on,
                               emit);
      } else if (a.F == 4) {
        apply_tile32<QP, 4, M>(a, hd, L, ncols, len, base, mu_p, nu_r, sp, sS, sz, sc, sf, pold, S, zold, yv, pv, on,
                               emit);
      } else {
#pragma unroll
        for (int qq = 0; qq < Q; ++qq) {
          const int s = threadIdx.x + qq * kCompute;
          on[qq] = false;
          yv[qq] = 0.f;
          pv[qq] = 0.f;
          if (s < len) {
            const int c = hcol_of(start, ncols, s);
            const int k = s - start[c];
            const int ctop = cn[c] & 0xffff, nk = cn[c] >> 16;
            if (k >= ctop) {
              on[qq] = true;
              float ru;
              yv[qq] = apply32<QP, M>(a, hd, L, c, s, k, ctop, nk, mu_p, nu_r, sp, sS, sz, sc, sf, pold, S, zold,
                                      pv[qq], ru);
              if (M) emit(qq, true, yv[qq], pv[qq], ru);
            }
          }
        }
      }
      // the stage is no longer read: hand it back to the producer
      __syncwarp();
      if (lane == 0) mbar_arrive(&P.empty[b]);
      if (!M) {
#pragma unroll
        for (int qq = 0; qq < Q; ++qq) {
          if (!on[qq]) continue;
          const int u = base + threadIdx.x + qq * kCompute;
          znew[u] = yv[qq];
          pnew[u] = pv[qq];
          df_addprod(dacc0, pv[qq], yv[qq]);
        }
      }
    } else {
      const float* sz = stage_stream(st, P.hcap, P.sfl, 2);
      float* sr = stage_stream(st, P.hcap, P.sfl, 3);
      {
        // 4 consecutive slots per thread: float4 in shared memory and global
        // (padding slots hold zeros in every stream and stay zero).  The
        // solution increment nu p is deferred to the next apply phase (or to
        // the reliable update), where p is streamed anyway.
        const int s0 = 4 * (int)threadIdx.x;
        if (s0 < len) {
          if (!a.x_in_apply) {
            const float4 p4 = *(const float4*)(stage_stream(st, P.hcap, P.sfl, 0) + s0);
            const float4 x4 = *(const float4*)(stage_stream(st, P.hcap, P.sfl, 1) + s0);
            *(float4*)(a.x32 + base + s0) = make_float4(__fmaf_rn(nu, p4.x, x4.x), __fmaf_rn(nu, p4.y, x4.y),
                                                        __fmaf_rn(nu, p4.z, x4.z), __fmaf_rn(nu, p4.w, x4.w));
          }
          const float4 z4 = *(const float4*)(sz + s0);
          const float4 r4 = *(const float4*)(sr + s0);
          const float4 ro = make_float4(__fmaf_rn(-nu, z4.x, r4.x), __fmaf_rn(-nu, z4.y, r4.y),
                                        __fmaf_rn(-nu, z4.z, r4.z), __fmaf_rn(-nu, z4.w, r4.w));
          *(float4*)(a.r32 + base + s0) = ro;
          if (QP == 2) {
            *(float4*)(sr + s0) = ro;
          } else {
            df_addprod(dacc0, ro.x, ro.x);
            df_addprod(dacc0, ro.y, ro.y);
            df_addprod(dacc0, ro.z, ro.z);
            df_addprod(dacc0, ro.w, ro.w);
          }
        }
      }
      if (QP == 2) {
        // Column tridiagonal solves entirely in shared memory: the p, x and z
        // streams of the stage are no longer needed, so they are refilled
        // (coalesced) with the Thomas factors tw, tib and the coefficients.
        csync();
        float* stw = stage_stream(st, P.hcap, P.sfl, 0);
        float* stib = stage_stream(st, P.hcap, P.sfl, 1);
        float* scf = stage_stream(st, P.hcap, P.sfl, 2);
        const int n4 = (len + 3) & ~3;
        for (int s = threadIdx.x; s < n4 + 4; s += kCompute) {
          if (s < n4) {
            stw[s] = a.tw32[base + s];
            stib[s] = a.tib32[base + s];
          }
          scf[s] = a.coef32[base + s];
        }
        csync();
        const unsigned char* hd = stage_hdr(st);
        const int ncols = ((const int*)hd)[0];
        const HdrLayout L = hdr_layout(ncols, a.F, len);
        const unsigned short* start = (const unsigned short*)(hd + L.o_start);
        const int* cn = (const int*)(hd + L.o_cn);
        for (int c = threadIdx.x; c < ncols; c += kCompute) {
          const int ctop = cn[c] & 0xffff, nk = cn[c] >> 16;
          const int b0 = start[c] + ctop, e0 = start[c] + nk;
          if (ctop == nk - 1) {
            stib[b0] = -0.5f * sr[b0] / scf[b0];
            continue;
          }
          // forward sweep: d'[k] = r[k] - w[k] d'[k-1], stored over w
          float d = sr[b0];
          stw[b0] = d;
          for (int s = b0 + 1; s < e0; ++s) {
            d = __fmaf_rn(-stw[s], d, sr[s]);
            stw[s] = d;
          }
          // backward sweep: u[k] = (d'[k] - coef[k+1] u[k+1]) / b'[k], stored over 1/b'
          float un = stw[e0 - 1] * stib[e0 - 1];
          stib[e0 - 1] = un;
          for (int s = e0 - 2; s >= b0; --s) {
            un = __fmaf_rn(-scf[s + 1], un, stw[s]) * stib[s];
            stib[s] = un;
          }
        }
        csync();
        // M^-1 r now in stib at wet levels; dry levels hold 0 in s32
        for (int s = threadIdx.x; s < len; s += kCompute) {
          const int c = hcol_of(start, ncols, s);
          const int k = s - start[c];
          const float sv = (k >= (cn[c] & 0xffff)) ? stib[s] : 0.f;
          a.s32[base + s] = sv;
          const float r = sr[s];
          df_addprod(dacc0, r, sv);
          df_addprod(NV == 2 ? dacc1 : dacc0, r, r);
        }
        csync();
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&P.empty[b]);
    }
    P.seq = q + 1;
  }
  if (cur >= 0) do_flush(cur, cur_enc);
  // The owner of each instance (the CTA holding its first tile) sums the
  // min(G, tiles) x 8 warp slots in a fixed order once every CTA has stored
  // them, restores the empty marks, and runs the finaliser.  Loads are issued
  // kPer at a time so that their latencies overlap.
  csync();
#ifdef SGPU_PHASE_TIMING
  const unsigned long long t_fin0 = globaltimer_ns();
#endif
  const int G = gridDim.x, nown = *P.nown;
  constexpr int kPer = 8 / NV;
  for (int o = 0; o < nown; ++o) {
    const int i = P.own[o];
    BInst* I = a.inst + i;
    const int t0 = I->t0, nt = I->t1 - I->t0;
    const int m8 = 8 * (nt < G ? nt : G);
    double v[NV];
#pragma unroll
    for (int vv = 0; vv < NV; ++vv) v[vv] = 0.0;
    volatile long long* base = (volatile long long*)(a.tpw + (size_t)t0 * 8 * kPwVals);
    for (int e0 = threadIdx.x; e0 < m8; e0 += kPer * kCompute) {
      long long bits[kPer][NV];
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const int e = e0 + k * kCompute;
#pragma unroll
        for (int vv = 0; vv < NV; ++vv) bits[k][vv] = e < m8 ? base[kPwVals * e + vv] : 0;
      }
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const int e = e0 + k * kCompute;
        if (e >= m8) continue;
#pragma unroll
        for (int vv = 0; vv < NV; ++vv) {
          double x;
          if (bits[k][vv] != kEmptyPartial) {
            base[kPwVals * e + vv] = kEmptyPartial;
            x = __longlong_as_double(bits[k][vv]);
          } else if (!take_partial((double*)(base + kPwVals * e + vv), lim, x)) {
            err = 1;
          }
          v[vv] += x;
        }
      }
    }
    csum<NV>(v, s_red);
    if (threadIdx.x == 0) fin(I, v);
  }
#ifdef SGPU_PHASE_TIMING
  // time the owners spend collecting and finalising (apply phase only)
  if (PH == 0 && nown > 0 && threadIdx.x == 0)
    atomicAdd((unsigned long long*)&a.ctl->phase_ns[0], globaltimer_ns() - t_fin0);
#endif
  if (err && threadIdx.x == 0) atomicCAS(&a.ctl->status, SGPU_OK, SGPU_TIMEOUT);
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
#ifndef SGPU_BATCH_MINB
#define SGPU_BATCH_MINB 3
#endif
// ONE: the one-pass form, a kernel of its own: its sweep keeps four
// double-float sums, three gathers per face and the new r, p and z live,
// which needs ~96 registers (2 CTAs per SM); the two-pass kernel fits in 72
// (3 CTAs per SM).
template <int QP, int ONE>
__global__ void __launch_bounds__(kThreads, ONE ? 2 : SGPU_BATCH_MINB) batch_kernel(BatchArgs a) {
  extern __shared__ __align__(128) unsigned char dyn[];
  __shared__ double s_red[4 * 8];
  __shared__ int s_flag;
  __shared__ int s_count;
  __shared__ int s_wsum[8];
  __shared__ int s_own[kListCap];
  __shared__ int s_nown;
  const int tid = threadIdx.x, F = a.F;
  const bool compute = tid < kCompute;
  SolveCtl* ctl = a.ctl;
  const long long lim = ctl->timeout_ns;

  Pipe P;
  P.hcap = a.hdr_cap;
  P.sfl = a.stream_floats;
  P.stage[0] = dyn;
  P.stage[1] = dyn + a.stage_bytes;
  P.full = (uint64_t*)(dyn + 2 * a.stage_bytes);
  P.empty = P.full + 2;
  P.list = (int*)(dyn + 2 * a.stage_bytes + 32);
  P.own = s_own;
  P.nown = &s_nown;
  P.count = &s_count;
  P.seq = 0;
  if (tid == 0) {
    mbar_init(&P.full[0], 1);
    mbar_init(&P.full[1], 1);
    mbar_init(&P.empty[0], 8);
    mbar_init(&P.empty[1], 8);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  TileSmem& sm = *(TileSmem*)P.stage[0];  // simple phases reuse stage 0 (no copies in flight then)

  // every partial-sum slot of this launch starts empty (a grid barrier orders
  // this before the first flush: in the set-up phases, or just below)
  for (size_t e = (size_t)blockIdx.x * blockDim.x + tid; e < (size_t)a.ntiles * 8 * kPwVals;
       e += (size_t)gridDim.x * blockDim.x)
    ((long long*)a.tpw)[e] = kEmptyPartial;
  if (!ld_volatile_int(&a.gflags[1]))
    if (!grid_sync(ctl, 5, [] {})) return;

  // ======================= setup of new instances =======================
  // gflags[1]: some instance needs its set-up phases (written by the host)
  if (ld_volatile_int(&a.gflags[1])) {
    auto is_setup = [&](int i) { return inst_state(a, i) == INST_SETUP; };
    if (compute) {
      // S1: conditioner / unscaled coefficients, FP32 copies, zero vectors
      for_tiles(a, is_setup, [&](int t, int i) {
        TileInfo ti;
        load_tile(a, t, ti, sm);
        const int len = ti.end - ti.base;
        if (QP == 1) {
          // the unscaled vertical coefficient of every wet slot first (one FP64
          // division per slot): a slot's diagonal also needs the coefficient
          // of the slot below, 2 Ac/(dzz[k+1] + dzz[k]), which is that slot's
          // own -- the same operands in the same order, so the same bits
          for (int s = tid; s < len; s += kCompute) {
            const int c = col_of(sm.start, sm.ncols, s);
            const int k = s - sm.start[c];
            const int u = ti.base + s;
            const int ctop = sm.ctop[c];
            const double dz = a.dzz64[u];
            const double Ac = a.colAc[ti.c0 + c];
            a.coef64[u] = k < ctop ? 0.0 : (k == ctop) ? Ac / dz : 2 * Ac / (dz + a.dzz64[u - 1]);
          }
          csync();
        }
        for (int s = tid; s < len; s += kCompute) {
          const int c = col_of(sm.start, sm.ncols, s);
          const int k = s - sm.start[c];
          const int u = ti.base + s;
          const int ctop = sm.ctop[c], nk = sm.nk[c];
          const bool act = k >= ctop;
          const double dz = a.dzz64[u];
          const double Ac = a.colAc[ti.c0 + c];
          a.r32[u] = 0.f;
          a.pa32[u] = 0.f;
          a.pb32[u] = 0.f;
          a.x32[u] = 0.f;
          a.z32[u] = 0.f;
          if (QP == 2) a.s32[u] = 0.f;
          else {
            a.r2_32[u] = 0.f;
            a.z2_32[u] = 0.f;
          }
          if (QP == 1) {
            double cc = 1.0;
            if (act) {
              double diag = 0.0;
              for (int f = 0; f < F; ++f) {
                const int kk = sm.fkk[c * F + f];
                if (k < (kk & 0xffff) || k >= (kk >> 16)) continue;
                diag += dz * a.face[(size_t)(ti.c0 + c) * F + f].D64;
              }
              const double ak = a.coef64[u];  // Ac/dzz or 2 Ac/(dzz + dzz above); scaled in S2
              if (ctop < nk - 1) {
                if (k == ctop) diag += 2 * ak + a.coef64[u + 1];
                else if (k == nk - 1) diag += ak;
                else diag += ak + a.coef64[u + 1];
              }
              if (diag <= 0) diag = 1;
              cc = sqrt(diag);
            }
            // c64 holds 1/c: one FP64 division per slot here instead of five
            // in the scaled coefficients (S2) and one in the rescale
            const double ic = 1.0 / cc;
            a.c64[u] = ic;
            a.cinv32[u] = (float)ic;
            a.fz32[u] = (float)(dz * ic);
            a.x64[u] = act ? a.q64[u] * cc : 0.0;
            a.b64[u] = act ? a.src64[u] * ic : 0.0;
          } else {
            double cf = 0.0;
            if (k == ctop) cf = Ac / dz;
            else if (k > ctop) cf = 2 * Ac / (dz + a.dzz64[u - 1]);
            a.coef64[u] = cf;
            a.coef32[u] = (float)cf;
            // per-slot copy of the edge levels' dzf*D that the inner apply streams
            for (int f = 0; f < F; ++f) {
              const int kk = sm.fkk[c * F + f];
              const bool on = act && k >= (kk & 0xffff) && k < (kk >> 16);
              a.fw32[(size_t)f * a.fw_stride + u] = on ? a.dzfD32[sm.fes[c * F + f] + k] : 0.f;
            }
            a.x64[u] = act ? a.q64[u] : 0.0;
            a.b64[u] = act ? a.src64[u] : 0.0;
          }
        }
        if (QP == 2) {
          csync();
          for (int c = tid; c < ti.c1 - ti.c0; c += kCompute)
            column_factor64(a, ti.base + sm.start[c], sm.ctop[c], sm.nk[c]);
        }
        csync();
      });
      // boundary (non-computational) slots of new instances: fixed values
      for (int i = 0; i < a.ninst; ++i) {
        const BInst& I = a.inst[i];
        if (ld_volatile_int(&I.state) != INST_SETUP) continue;
        for (int u = I.s1 + blockIdx.x * kCompute + tid; u < I.s2; u += gridDim.x * kCompute) {
          a.x64[u] = a.q64[u];
          a.b64[u] = 0.0;
          a.r32[u] = 0.f;
          a.pa32[u] = 0.f;
          a.pb32[u] = 0.f;
          a.z32[u] = 0.f;
          if (QP == 2) a.s32[u] = 0.f;
          else {
            a.r2_32[u] = 0.f;
            a.z2_32[u] = 0.f;
          }
          if (QP == 1) {
            const double ic = 1.0 / a.cin64[u];
            a.c64[u] = ic;
            a.cinv32[u] = (float)ic;
          }
        }
      }
    }
    if (!grid_sync(ctl, 5, [] {})) return;

    // S2 (qprecond 1): FP64 scaled coefficients (QCoefficients 3427-3452) and
    // their FP32 vertical copy
    if (QP == 1) {
      if (compute)
        for_tiles(a, is_setup, [&](int t, int i) {
          TileInfo ti;
          load_tile(a, t, ti, sm);
          const int len = ti.end - ti.base;
          for (int s = tid; s < len; s += kCompute) {
            const int c = col_of(sm.start, sm.ncols, s);
            const int k = s - sm.start[c];
            const int u = ti.base + s;
            const int ctop = sm.ctop[c];
            const double Ac = a.colAc[ti.c0 + c];
            const double dz = a.dzz64[u];
            const double icu = a.c64[u];  // 1/c
            const double ak = a.coef64[u];  // Ac/dzz or 2 Ac/(dzz + dzz above), from S1
            double cf = 0.0;
            if (k == ctop) cf = ak * icu;
            else if (k > ctop) cf = ak * (icu * a.c64[u - 1]);
            a.coef64[u] = cf;
            a.coef32[u] = (float)cf;
            for (int f = 0; f < F; ++f) {
              const int kk = sm.fkk[c * F + f];
              double v = 0.0;
              if (k >= ctop && k >= (kk & 0xffff) && k < (kk >> 16))
                v = dz * a.face[(size_t)(ti.c0 + c) * F + f].D64 * (icu * a.c64[sm.fns[c * F + f] + k]);
              a.fc64[(size_t)F * u + f] = v;
              // the FP32 weight the inner apply uses: (dzz/c_u) * (D * (1/c_n)), as formed
              // from the FP32 copies (0 where the face does not couple the level)
              float w = 0.f;
              if (k >= ctop && k >= (kk & 0xffff) && k < (kk >> 16))
                w = a.fz32[u] * (a.face[(size_t)(ti.c0 + c) * F + f].D * a.cinv32[sm.fns[c * F + f] + k]);
              a.fw32[(size_t)f * a.fw_stride + u] = w;
            }
          }
          csync();
        });
      if (!grid_sync(ctl, 6, [] {})) return;
    }

    // S3: initial FP64 residual, first preconditioned residual, alpha0, eps0
    if (compute)
      for_tiles_reduce<2>(a, s_red, &s_flag, is_setup,
          [&](int t, int i, double (&acc)[2]) {
            TileInfo ti;
            load_tile(a, t, ti, sm);
            const int len = ti.end - ti.base;
            for (int s = tid; s < len; s += kCompute) {
              const int c = col_of(sm.start, sm.ncols, s);
              const int k = s - sm.start[c];
              const int u = ti.base + s;
              const int ctop = sm.ctop[c], nk = sm.nk[c];
              if (k < ctop) continue;
              const double r = a.b64[u] - apply64<QP>(a, sm, c, u, k, ctop, nk, a.x64);
              const float rf = (float)r;
              a.r32[u] = rf;
              if (QP == 2) acc[1] += r * r;
              else acc[0] += f2d(rf) * f2d(rf);
            }
            if (QP == 2) {
              csync();
              for (int c = tid; c < ti.c1 - ti.c0; c += kCompute)
                column_solve32(a, a.r32, 0, ti.base + sm.start[c], sm.ctop[c], sm.nk[c]);
              csync();
              for (int u = ti.base + tid; u < ti.end; u += kCompute) acc[0] += f2d(a.r32[u]) * f2d(a.s32[u]);
            }
            csync();
          },
          [&](BInst* I, const double* tot) {
            double alpha0 = tot[0];
            if (!I->resnorm) alpha0 = 1;
            const double eps0 = (QP == 2) ? tot[1] : alpha0;
            I->alpha = tot[0];
            I->eps0 = eps0;
            I->eps = eps0;
            I->eps_ref = eps0;
            I->mu = 0.0;
            I->nu = 0.0;
            I->nu_x = 0.0;
            I->n = 0;
            I->nrel = 0;
            I->flags = 0;
            I->par = 0;
            I->status = SGPU_OK;
            I->state = (I->maxiters <= 0 || eps0 == 0) ? INST_DONE : INST_RUN;
          });
    if (!grid_sync(ctl, 7, [&] {
          if (tid == 0) {
            int any = 0;
            for (int i = 0; i < a.ninst; ++i) any |= (a.inst[i].state == INST_RUN);
            a.gflags[3] = any;
            __threadfence();
          }
        }))
      return;
  }

  // ============================ iterations ==============================
  // A running instance takes part in global iteration it unless its stride
  // skips it (the same decision in every CTA: it and the stride are uniform);
  // a skipped iteration leaves the instance's state untouched, so its own
  // iteration sequence, and its bits, do not depend on the stride.
  int it_now = 0;
  auto is_run = [&](int i) {
    if (inst_state(a, i) != INST_RUN) return false;
    const int st = ld_volatile_int(&a.inst[i].stride);
    return st <= 1 || it_now % st == 0;
  };
  for (int it = 0; it < a.max_iters_chunk; ++it) {
    if (!ld_volatile_int(&a.gflags[3])) break;
    it_now = it;

    if (QP != 2 && ONE) {
      // ---- one pass: r_j = r - nu z, x += nu p_old, p_j = r_j + mu p_old,
      //      z_j = A p_j; p.z, r.r, r.z, z.z ----
      // CG with the two reductions of an iteration merged (the residual step
      // of iteration j-1 is taken in the sweep of iteration j): nu_j =
      // r_j.r_j / p_j.z_j as in the two-pass form, and the next mu from
      // |r_j - nu_j z_j|^2 = r.r - 2 nu r.z + nu^2 z.z of this sweep's own
      // vectors.  The convergence test sees r_j.r_j one sweep after the
      // two-pass form would, so a solve takes one sweep more than its
      // iteration count.
      build_list(a, P, is_run, s_wsum);
      pipelined_phase<QP, 2>(a, P, s_red, &s_flag, lim, [&](BInst* In, const double* tot) {
        const double pz = tot[0], rr = tot[1], rz = tot[2], zz = tot[3];
        const bool moved = In->nu != 0.0;  // this sweep took the pending step (not the first, nor one after a refresh)
        const int n = In->n + (moved ? 1 : 0);
        In->n = n;
        In->nu_x = 0.0;
        const double eps = rr;
        In->eps = eps;
        int flags = 0;
        if (!isfinite(rr) || !isfinite(pz)) {
          In->status = SGPU_BREAKDOWN;
          In->state = INST_DONE;
          flags = 2;
        } else if (moved) {
          if (eps == 0) {
            In->state = INST_DONE;
            flags = 2;
          } else if (eps < In->tol2 * In->eps0 || eps < a.delta2 * In->eps_ref) {
            flags = 1;  // verify / refresh with the FP64 true residual
          } else if (n >= In->maxiters) {
            In->status = SGPU_MAXITER;
            In->state = INST_DONE;
            flags = 2;
          }
          if (flags == 1 && n >= In->maxiters) flags = 1 | 4;  // last chance: verify, else stop
        }
        if (flags == 0) {
          const double nu = rr / pz;
          double rnext = rr - 2.0 * nu * rz + nu * nu * zz;
          if (!(rnext > 0.0)) rnext = 0.0;  // cancellation at convergence: restart the direction
          if (!isfinite(nu)) {
            In->status = SGPU_BREAKDOWN;
            In->state = INST_DONE;
            flags = 2;
          } else {
            In->alpha = rr;
            In->nu = nu;
            In->mu = rnext / rr;
            In->par ^= 1;  // the sweep wrote the other buffers of p, r and z
          }
        } else if (flags & 1) {
          // refresh: this sweep's direction is dropped.  R2 writes the true
          // residual over the residual this sweep read (buffer par, kept), and
          // the next sweep forms p_j again from it with mu = rho_true / rho_{j-1}
          // and the direction p_{j-1} still in buffer par; x32 holds x_j, so
          // nothing is pending.
          In->alpha_prev = In->alpha;
          In->nu = 0.0;
        }
        In->flags = flags;
        if (flags) atomicOr(&a.gflags[0], 1);
      });
      if (!grid_sync(ctl, 2, [&] {
            if (tid == 0) {
              a.gflags[2] = a.gflags[0];
              a.gflags[0] = 0;
              __threadfence();
            }
          }))
        return;
    } else {
      // ---- A: p_new = S + mu p_old (on the fly), z = A p_new, p.z ----
      build_list(a, P, is_run, s_wsum);
      pipelined_phase<QP, 0>(a, P, s_red, &s_flag, lim, [&](BInst* In, const double* tot) {
        In->nu_x = 0.0;  // this phase's tiles added the pending solution increment
        const double alpha = In->alpha;
        In->alpha_prev = alpha;
        In->mu = 1 / alpha;  // mu = 1/alpha before nu (2484-2485)
        const double nu = alpha / tot[0];
        In->nu = nu;
        In->par ^= 1;
        if (!isfinite(nu)) {
          In->status = SGPU_BREAKDOWN;
          In->flags = 2;  // final merge
          In->state = INST_DONE;
          atomicOr(&a.gflags[0], 1);
        }
      });
      if (!grid_sync(ctl, 1, [] {})) return;

      // ---- B: x32 += nu p, r -= nu z, preconditioner, r.s, r.r ----
      build_list(a, P, is_run, s_wsum);
      pipelined_phase<QP, 1>(a, P, s_red, &s_flag, lim, [&](BInst* In, const double* tot) {
        const double alpha = tot[0];
        const double mu = In->mu * alpha;  // mu *= alpha (2498/2509)
        In->mu = mu;
        In->alpha = alpha;
        In->nu_x = a.x_in_apply ? In->nu : 0.0;  // x32 += nu p now pending (next apply phase or R1)
        const double eps = (QP == 2) ? tot[1] : alpha;
        In->eps = eps;
        const int n = In->n + 1;
        In->n = n;
        int flags = 0;
        if (!isfinite(alpha) || !isfinite(mu)) {
          In->status = SGPU_BREAKDOWN;
          In->state = INST_DONE;
          flags = 2;
        } else if (eps == 0) {
          In->state = INST_DONE;
          flags = 2;
        } else if (eps < In->tol2 * In->eps0 || eps < a.delta2 * In->eps_ref) {
          flags = 1;  // verify / refresh with the FP64 true residual
        } else if (n >= In->maxiters) {
          In->status = SGPU_MAXITER;
          In->state = INST_DONE;
          flags = 2;
        }
        if (flags == 1 && n >= In->maxiters) flags = 1 | 4;  // last chance: verify, else stop
        In->flags = flags;
        if (flags) atomicOr(&a.gflags[0], 1);
      });
      if (!grid_sync(ctl, 2, [&] {
            if (tid == 0) {
              a.gflags[2] = a.gflags[0];
              a.gflags[0] = 0;
              __threadfence();
            }
          }))
        return;
    }

    if (ld_volatile_int(&a.gflags[2])) {
      auto flagged = [&](int i) { return inst_flags(a, i) != 0; };
      // ---- R1: x64 += x32 (+ the pending nu p), x32 = 0 for flagged instances ----
      if (compute)
        for_tiles(a, flagged, [&](int t, int i) {
          const TileDesc d = a.tiles[t];
          const BInst& I = a.inst[i];
          const float nux = (float)(*(volatile const double*)&I.nu_x);
          const float* p = ld_volatile_int(&I.par) ? a.pb32 : a.pa32;  // the direction of the last update phase
          for (int u = d.base + tid; u < d.base + d.nslots; u += kCompute) {
            const float x = nux != 0.f ? __fmaf_rn(nux, p[u], a.x32[u]) : a.x32[u];
            a.x64[u] += f2d(x);
            a.x32[u] = 0.f;
          }
        });
      if (!grid_sync(ctl, 3, [] {})) return;
      // ---- R2: FP64 true residual for instances that verify / refresh ----
      if (compute)
        for_tiles_reduce<2>(a, s_red, &s_flag, flagged,
            [&](int t, int i, double (&acc)[2]) {
              if (!(inst_flags(a, i) & 1)) return;  // final merge only: counted, nothing to compute
              TileInfo ti;
              load_tile(a, t, ti, sm);
              const int len = ti.end - ti.base;
              float* rout = rbuf(a, ld_volatile_int(&a.inst[i].par));  // the residual the next sweep reads
              for (int s = tid; s < len; s += kCompute) {
                const int c = col_of(sm.start, sm.ncols, s);
                const int k = s - sm.start[c];
                const int u = ti.base + s;
                const int ctop = sm.ctop[c], nk = sm.nk[c];
                if (k < ctop) continue;
                const double r = a.b64[u] - apply64<QP>(a, sm, c, u, k, ctop, nk, a.x64);
                rout[u] = (float)r;
                if (QP == 2) acc[1] += r * r;
                else acc[0] += r * r;
              }
              if (QP == 2) {
                csync();
                for (int c = tid; c < ti.c1 - ti.c0; c += kCompute)
                  column_solve32(a, a.r32, 0, ti.base + sm.start[c], sm.ctop[c], sm.nk[c]);
                csync();
                for (int u = ti.base + tid; u < ti.end; u += kCompute) acc[0] += f2d(a.r32[u]) * f2d(a.s32[u]);
              }
              csync();
            },
            [&](BInst* In, const double* tot) {
              In->nu_x = 0.0;  // R1 added the pending solution increment
              if (!(In->flags & 1)) {
                In->flags = 0;
                return;
              }
              const double alpha = tot[0];
              const double eps = (QP == 2) ? tot[1] : alpha;
              In->nrel += 1;
              In->eps = eps;
              In->eps_ref = eps;
              if (eps < In->tol2 * In->eps0 || eps == 0) {
                In->state = INST_DONE;
              } else if (In->flags & 4) {
                In->status = SGPU_MAXITER;
                In->state = INST_DONE;
              } else {
                In->mu = alpha / In->alpha_prev;  // beta from the true residual
                In->alpha = alpha;
              }
              In->flags = 0;
            });
      if (!grid_sync(ctl, 4, [&] {
            if (tid == 0) {
              int any = 0;
              for (int i = 0; i < a.ninst; ++i) any |= (a.inst[i].state == INST_RUN);
              a.gflags[3] = any;
              __threadfence();
            }
          }))
        return;
    }
  }
}

// q64 := the solution of an instance's computational slots (warm start for a
// re-submission, and the unscaled result for download)
__global__ void finalize_q_kernel(const double* __restrict__ x64, const double* __restrict__ c64,
                                  double* __restrict__ q64, int s0, int n, int scaled) {
  for (int u = s0 + blockIdx.x * blockDim.x + threadIdx.x; u < s0 + n; u += gridDim.x * blockDim.x)
    q64[u] = scaled ? x64[u] * c64[u] : x64[u];  // c64 holds 1/c
}

}  // namespace sgpu

namespace sgpu {
// ---------------------------------------------------------------------------
// host side: the batch engine
// ---------------------------------------------------------------------------
struct Range {
  long long off = 0, len = 0;
};

// Runs fn(begin, end) over [0, n) on up to 8 host threads (one per `grain`
// items), for the per-column copies between caller rows and pinned staging.
template <class Fn>
static void host_split(long long n, long long grain, Fn&& fn) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<long long>(std::min(hw, 8u), std::max(1LL, n / std::max(1LL, grain)));
  if (nt <= 1) {
    fn(0LL, n);
    return;
  }
  std::vector<std::thread> th;
  const long long chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const long long b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back([&fn, b, e] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

// first-fit allocator over [0, cap) in units of `unit`
struct Arena {
  long long cap = 0, unit = 1;
  std::vector<Range> freel;
  void init(long long c, long long u = 1) {
    unit = u;
    cap = c / u * u;
    freel.assign(1, Range{0, cap});
  }
  long long round(long long n) const { return (n + unit - 1) / unit * unit; }
  long long alloc(long long n) {
    n = round(std::max(n, 1LL));
    for (size_t i = 0; i < freel.size(); ++i)
      if (freel[i].len >= n) {
        long long o = freel[i].off;
        freel[i].off += n;
        freel[i].len -= n;
        if (freel[i].len == 0) freel.erase(freel.begin() + i);
        return o;
      }
    return -1;
  }
  void release(long long off, long long n) {
    n = round(std::max(n, 1LL));
    freel.push_back(Range{off, n});
    std::sort(freel.begin(), freel.end(), [](const Range& x, const Range& y) { return x.off < y.off; });
    std::vector<Range> m;
    for (auto& r : freel) {
      if (!m.empty() && m.back().off + m.back().len == r.off) m.back().len += r.len;
      else m.push_back(r);
    }
    freel.swap(m);
  }
  long long free_total() const {
    long long s = 0;
    for (auto& r : freel) s += r.len;
    return s;
  }
};

struct HostTile {
  int c0, c1;          // relative computational columns
  int base, nslots;    // relative slots
  int hdr, hdr_bytes;  // relative header bytes
};

struct HostInst {
  bool live = false;
  int id = -1;
  long long s_off = 0, n3 = 0, n3c = 0;  // slots (n3 includes tile padding)
  long long c_off = 0, ncomp = 0;        // columns
  long long e_off = 0, ne3 = 0;          // edge slots
  long long h_off = 0, h_bytes = 0;      // header bytes
  int Nc = 0;
  std::vector<int> dev2cell, Nk, ctop, coff;  // device column -> cell; per cell Nk/ctop; device column -> relative slot
  std::vector<HostTile> tiles;
  long long unk = 0;                          // pressure unknowns: sum of Nk - ctop over computational cells
  int last_iters = 0;                         // iterations of its last finished solve (0 = none yet)
};

}  // namespace sgpu

using namespace sgpu;

struct sgpu_batch {
  int device = 0;
  int qprecond = 1;
  int F = 3;
  cudaStream_t stream = nullptr;   // launches
  cudaStream_t ustream = nullptr;  // uploads of added / re-submitted problems and result downloads, which touch
                                   // only problems outside the launch in flight
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  long long timeout_ns = 2000000000LL;
  int grid_override = 0;
  int tile_slots = kBTSlots;  // storage slots per tile for instances added from now on
  double delta = 0.01;
  long long max_slots = 0, max_cols = 0, max_eslots = 0, max_hdr = 0;
  int max_inst = 0, max_tiles = 0;
  Arena slots, cols, eslots, hdrs;
  std::vector<HostInst> inst;
  BInst* h_inst = nullptr;         // pinned, max_inst entries: the host's view
  BInst* h_inst_up = nullptr;      // pinned: the table a launch uploads (a copy taken when it is enqueued)
  BInst* h_inst_dev = nullptr;     // pinned: the table a launch writes back
  bool inflight = false;           // a launch is enqueued and not yet waited for
  std::vector<int> launched;       // problems that launch runs (their rows of h_inst_dev are taken after it)
  int launched_ninst = 0;
  TileDesc* h_tiles = nullptr;     // pinned, max_tiles entries
  int* h_tinst = nullptr;          // pinned
  int* h_gflags = nullptr;         // pinned [4]
  double* h_stage = nullptr;       // pinned staging for re-submitted right-hand sides
  long long h_stage_n = 0;
  std::vector<int> n_before;
  // CUDA graph of the launch sequence (tables in, kernel, instance table out)
  bool use_graph = false, graph_failed = false;
  cudaGraphExec_t gexec = nullptr;
  int g_ntiles = -1, g_ninst = -1, g_grid = -1, g_chunk = -1;
  // the captured launch's by-value arguments that the key above does not fix
  int g_stage = -1, g_hdr = -1, g_sfl = -1, g_fusion = -1;
  double g_delta = -1.0;
  long long graph_launches = 0;
  // device
  std::vector<void*> allocs;
  BatchArgs a{};
  TileDesc* d_tiles = nullptr;
  int* d_tile_inst = nullptr;
  unsigned char* d_hdrs = nullptr;
  BCol* d_col = nullptr;
  BFace* d_face = nullptr;
  double* d_colAc = nullptr;
  double *d_dzz64 = nullptr, *d_src64 = nullptr, *d_q64 = nullptr, *d_cin64 = nullptr, *d_dzfD64 = nullptr;
  BInst* d_inst = nullptr;
  SolveCtl* d_ctl = nullptr;
  int* d_gflags = nullptr;
  SolveCtl* h_ctl = nullptr;
  int ntiles = 0;
  double last_ms = 0.0;
  long long last_work = 0;
  bool attr_set[3][2] = {};
  int streams = 4;                    // FP32 streams per pipeline stage
  int x_in_apply = 1;                 // the solution update's place (BatchArgs::x_in_apply)
  int fusion = 1;                     // sgpu_batch_set_fusion's form: 0, 1 or 2 (one pass; qprecond 0/1)
  int dyn_smem = kDynSmem;            // dynamic shared memory of the kernel
};

static int bfail(sgpu_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(call)                                                                                          \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? SGPU_OOM : SGPU_CUDA_ERROR, "%s: %s (line %d)", #call, \
                   cudaGetErrorString(e_), __LINE__);                                                      \
  } while (0)

template <class T>
static int balloc(sgpu_batch* b, T** p, size_t n) {
  void* v = nullptr;
  BCK(cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T)));
  b->allocs.push_back(v);
  *p = (T*)v;
  return SGPU_OK;
}

namespace {
struct Guard {
  int prev = -1;
  explicit Guard(int d) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(d);
  }
  ~Guard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

const void* kernel_of(int qp, bool one) {
  if (one) return qp == 1 ? (const void*)batch_kernel<1, 1> : (const void*)batch_kernel<0, 1>;
  return qp == 1 ? (const void*)batch_kernel<1, 0>
                 : qp == 2 ? (const void*)batch_kernel<2, 0> : (const void*)batch_kernel<0, 0>;
}
}  // namespace

static int batch_max_grid(sgpu_batch* b, bool one) {
  const void* fn = kernel_of(b->qprecond, one);
  if (!b->attr_set[b->qprecond][one]) {
    // the largest stage configuration any batch may use (the one-pass form's
    // 5 + F streams at 8 faces), so that batches of different face counts and
    // forms sharing the kernel never find the limit too low
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem_bytes(5 + kMaxF)) !=
        cudaSuccess)
      return 0;
    b->attr_set[b->qprecond][one] = true;
  }
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kThreads, b->dyn_smem) != cudaSuccess) return 0;
  return sms * per;
}

extern "C" {

int sgpu_batch_create(int device, int qprecond, int maxfaces, long long max_slots, long long max_cols,
                      long long max_edge_slots, int max_instances, sgpu_batch** out) {
  if (!out || qprecond < 0 || qprecond > 2 || maxfaces < 1 || maxfaces > kMaxF || max_slots <= 0 ||
      max_cols <= 0 || max_instances <= 0 || max_slots > 0x7ffffff0LL || max_edge_slots > 0x7ffffff0LL)
    return SGPU_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return SGPU_NO_DEVICE;
  if (device < 0 || device >= ndev) return SGPU_BAD_ARG;
  sgpu_batch* b = new sgpu_batch();
  *out = b;
  b->device = device;
  b->qprecond = qprecond;
  b->F = maxfaces;
  b->streams = 4 + maxfaces;
  b->dyn_smem = dyn_smem_bytes(b->streams);
  // tiles are 4-slot aligned: reserve room for the padding (< 4 slots per tile)
  const long long tiles_est = max_cols + max_slots / kBTSlots + 2LL * max_instances + 2;
  b->max_slots = std::min(0x7ffffff0LL, max_slots + 4 * std::min(tiles_est, max_slots) + 8LL * max_instances + 16);
  b->max_cols = max_cols;
  b->max_eslots = std::max(1LL, max_edge_slots);
  b->max_inst = max_instances;
  b->max_tiles = (int)std::min<long long>(0x7fffffff, tiles_est);
  // header bytes: per tile 16 + 3 x 16 padding, per column 2 + 4, per column-face 16
  b->max_hdr = 80LL * (b->max_tiles + 1) + (long long)max_cols * (8 + 16LL * maxfaces) + 16;
  if (b->max_hdr > 0x7ffffff0LL) return bfail(b, SGPU_BAD_ARG, "header arena too large");
  b->slots.init(b->max_slots, 4);
  b->cols.init(max_cols);
  b->eslots.init(b->max_eslots);
  b->hdrs.init(b->max_hdr, 16);
  b->inst.resize(max_instances);
  b->n_before.assign(max_instances, 0);
  Guard g(device);
  BCK(cudaMallocHost((void**)&b->h_inst, sizeof(BInst) * max_instances));
  BCK(cudaMallocHost((void**)&b->h_inst_up, sizeof(BInst) * max_instances));
  BCK(cudaMallocHost((void**)&b->h_inst_dev, sizeof(BInst) * max_instances));
  std::memset(b->h_inst, 0, sizeof(BInst) * max_instances);
  BCK(cudaMallocHost((void**)&b->h_tiles, sizeof(TileDesc) * ((size_t)b->max_tiles + 1)));
  std::memset(b->h_tiles, 0xff, sizeof(TileDesc) * ((size_t)b->max_tiles + 1));
  BCK(cudaMallocHost((void**)&b->h_tinst, sizeof(int) * ((size_t)b->max_tiles + 1)));
  BCK(cudaMallocHost((void**)&b->h_gflags, 4 * sizeof(int)));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCK(cudaStreamCreateWithFlags(&b->ustream, cudaStreamNonBlocking));
  BCK(cudaEventCreate(&b->ev0));
  BCK(cudaEventCreate(&b->ev1));
  BCK(cudaMallocHost((void**)&b->h_ctl, sizeof(SolveCtl)));
  const size_t S = (size_t)b->max_slots + 8, E = (size_t)b->max_eslots + 8, Cn = (size_t)max_cols + 1;
  int rc;
  BatchArgs& a = b->a;
  a.F = maxfaces;
  if ((rc = balloc(b, &b->d_tiles, (size_t)b->max_tiles + 1))) return rc;
  if ((rc = balloc(b, &b->d_tile_inst, (size_t)b->max_tiles + 1))) return rc;
  if ((rc = balloc(b, &b->d_hdrs, (size_t)b->max_hdr))) return rc;
  if ((rc = balloc(b, &b->d_col, Cn))) return rc;
  if ((rc = balloc(b, &b->d_face, Cn * maxfaces))) return rc;
  if ((rc = balloc(b, &b->d_colAc, Cn))) return rc;
  if ((rc = balloc(b, &b->d_dzz64, S))) return rc;
  if ((rc = balloc(b, &b->d_src64, S))) return rc;
  if ((rc = balloc(b, &b->d_q64, S))) return rc;
  if ((rc = balloc(b, &b->d_cin64, S))) return rc;
  if ((rc = balloc(b, &b->d_dzfD64, E))) return rc;
  if ((rc = balloc(b, &a.c64, S))) return rc;
  if ((rc = balloc(b, &a.coef64, S))) return rc;
  if (qprecond == 1 && (rc = balloc(b, &a.fc64, S * maxfaces))) return rc;
  if ((rc = balloc(b, &a.x64, S))) return rc;
  if ((rc = balloc(b, &a.b64, S))) return rc;
  if ((rc = balloc(b, &a.fz32, S))) return rc;
  {
    // one array per face, each starting on a 128-byte boundary: the bulk copies
    // of a tile's weights need 16-byte aligned sources
    const size_t FS = (S + 31) & ~(size_t)31;
    a.fw_stride = (long long)FS;
    if ((rc = balloc(b, &a.fw32, FS * (size_t)maxfaces))) return rc;
    BCK(cudaMemsetAsync(a.fw32, 0, FS * (size_t)maxfaces * sizeof(float), b->stream));
  }
  if ((rc = balloc(b, &a.cinv32, S))) return rc;
  if ((rc = balloc(b, &a.coef32, S))) return rc;
  if ((rc = balloc(b, &a.dzfD32, E))) return rc;
  if (qprecond == 2) {
    if ((rc = balloc(b, &a.tw32, S))) return rc;
    if ((rc = balloc(b, &a.tib32, S))) return rc;
    if ((rc = balloc(b, &a.s32, S))) return rc;
  }
  if ((rc = balloc(b, &a.r32, S))) return rc;
  if ((rc = balloc(b, &a.pa32, S))) return rc;
  if ((rc = balloc(b, &a.pb32, S))) return rc;
  if ((rc = balloc(b, &a.x32, S))) return rc;
  if ((rc = balloc(b, &a.z32, S))) return rc;
  if (qprecond != 2) {
    if ((rc = balloc(b, &a.r2_32, S))) return rc;
    if ((rc = balloc(b, &a.z2_32, S))) return rc;
  }
  if ((rc = balloc(b, &a.tpart, 2 * ((size_t)b->max_tiles + 1)))) return rc;
  if ((rc = balloc(b, &a.tpw, 8 * kPwVals * ((size_t)b->max_tiles + 1)))) return rc;
  if ((rc = balloc(b, &b->d_inst, (size_t)max_instances))) return rc;
  if ((rc = balloc(b, &b->d_ctl, 1))) return rc;
  if ((rc = balloc(b, &b->d_gflags, 4))) return rc;
  // padding slots are copied by the bulk copies but never used: keep them finite
  float* f32s[] = {a.fz32, a.cinv32, a.coef32, a.r32, a.pa32, a.pb32, a.x32, a.z32, a.r2_32, a.z2_32, a.s32,
                   a.tw32, a.tib32};
  for (float* p : f32s)
    if (p) BCK(cudaMemsetAsync(p, 0, S * sizeof(float), b->stream));
  BCK(cudaMemsetAsync(a.coef64, 0, S * sizeof(double), b->stream));
  BCK(cudaMemsetAsync(b->d_cin64, 0, S * sizeof(double), b->stream));
  BCK(cudaMemsetAsync(b->d_inst, 0, sizeof(BInst) * max_instances, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  a.tiles = b->d_tiles;
  a.tile_inst = b->d_tile_inst;
  a.hdrs = b->d_hdrs;
  a.col = b->d_col;
  a.face = b->d_face;
  a.colAc = b->d_colAc;
  a.dzz64 = b->d_dzz64;
  a.src64 = b->d_src64;
  a.q64 = b->d_q64;
  a.cin64 = b->d_cin64;
  a.dzfD64 = b->d_dzfD64;
  a.inst = b->d_inst;
  a.ctl = b->d_ctl;
  a.gflags = b->d_gflags;
  return SGPU_OK;
}

int sgpu_batch_destroy(sgpu_batch* b) {
  if (!b) return SGPU_BAD_ARG;
  {
    Guard g(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->ustream) cudaStreamSynchronize(b->ustream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (void* p : b->allocs) cudaFree(p);
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->h_inst) cudaFreeHost(b->h_inst);
    if (b->h_inst_up) cudaFreeHost(b->h_inst_up);
    if (b->h_inst_dev) cudaFreeHost(b->h_inst_dev);
    if (b->h_tiles) cudaFreeHost(b->h_tiles);
    if (b->h_tinst) cudaFreeHost(b->h_tinst);
    if (b->h_gflags) cudaFreeHost(b->h_gflags);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->ustream) cudaStreamDestroy(b->ustream);
  }
  delete b;
  return SGPU_OK;
}

const char* sgpu_batch_last_error(const sgpu_batch* b) { return b ? b->err.c_str() : "null batch"; }

long long sgpu_batch_bytes_per_request(int qprecond, int maxfaces, long long n3, long long ncols,
                                       long long nedge_slots) {
  // device bytes an instance occupies (layout of sgpu_batch_create's arrays)
  long long per_slot = 8 * 8 + 4 * 8 + 4LL * maxfaces + (qprecond == 1 ? 8LL * maxfaces : 0) + (qprecond == 2 ? 12 : 0);
  long long per_col = (long long)sizeof(BCol) + (long long)sizeof(BFace) * maxfaces + 8 + 8 + 16LL * maxfaces;
  long long per_eslot = 12;
  const long long tiles = ncols / 16 + n3 / kBTSlots + 2;
  return per_slot * (n3 + 4 * tiles) + per_col * ncols + per_eslot * nedge_slots + (96 + 128) * tiles;
}

int sgpu_batch_add(sgpu_batch* b, const sgpu_grid_desc* g, const int* ctop, const double* const* dzz,
                   const double* const* dzf, const double* D, const double* const* q, const double* const* src,
                   const double* const* c, double qepsilon, int qmaxiters, double resnorm, int* id_out) {
  if (!b || !g || !ctop || !dzz || !dzf || !D || !q || !src || !id_out) return SGPU_BAD_ARG;
  if (g->maxfaces != b->F) return bfail(b, SGPU_BAD_ARG, "maxfaces %d differs from the batch's %d", g->maxfaces, b->F);
  const int Nc = g->Nc, Ne = g->Ne, F = g->maxfaces;
  const int* cd = g->celldist;
  if (Nc <= 0 || !cd || !(cd[0] == 0 && cd[0] <= cd[1] && cd[1] <= cd[2] && cd[2] <= Nc) || cd[1] == 0)
    return bfail(b, SGPU_BAD_GRID, "celldist must satisfy 0 = c0 < c1 <= c2 <= Nc");
  if (g->Nkmax > kTileCap) return bfail(b, SGPU_BAD_GRID, "Nkmax %d exceeds %d", g->Nkmax, kTileCap);
  int id = -1;
  for (int i = 0; i < b->max_inst; ++i)
    if (!b->inst[i].live) {
      id = i;
      break;
    }
  if (id < 0) return bfail(b, SGPU_OOM, "no free instance slot (max %d)", b->max_inst);
  HostInst H;
  H.live = true;
  H.id = id;
  H.Nc = Nc;
  H.Nk.assign(g->Nk, g->Nk + Nc);
  H.ctop.assign(ctop, ctop + Nc);
  // device order: cellp[0..c2) then the rest
  std::vector<int> c2d(Nc, -1);
  for (int t = 0; t < cd[2]; ++t) {
    const int i = g->cellp[t];
    if (i < 0 || i >= Nc || c2d[i] >= 0) return bfail(b, SGPU_BAD_GRID, "cellp invalid or repeated");
    c2d[i] = (int)H.dev2cell.size();
    H.dev2cell.push_back(i);
  }
  for (int i = 0; i < Nc; ++i)
    if (c2d[i] < 0) {
      c2d[i] = (int)H.dev2cell.size();
      H.dev2cell.push_back(i);
    }
  for (int j = 0; j < Nc; ++j) {
    const int i = H.dev2cell[j];
    if (g->Nk[i] < 1 || g->Nk[i] > g->Nkmax || ctop[i] < 0 || ctop[i] >= g->Nk[i])
      return bfail(b, SGPU_BAD_GRID, "Nk/ctop out of range at cell %d", i);
    if (g->nfaces[i] < 1 || g->nfaces[i] > F) return bfail(b, SGPU_BAD_GRID, "nfaces out of range at cell %d", i);
  }
  // tiles over the computational columns: <= kBTSlots slots, <= kBTCols columns,
  // <= kBTFaces column-faces; every tile starts on a 4-slot boundary
  const int maxc = std::min(kBTCols, kBTFaces / F);
  const int cap = std::max(b->tile_slots, g->Nkmax);  // a column always fits a tile
  H.coff.assign(Nc + 1, 0);
  long long acc = 0, hacc = 0;
  {
    int j = 0;
    while (j < cd[1]) {
      HostTile T;
      T.c0 = j;
      T.base = (int)acc;
      int len = 0;
      while (j < cd[1] && j - T.c0 < maxc && len + g->Nk[H.dev2cell[j]] <= cap) {
        H.coff[j] = (int)(acc + len);
        len += g->Nk[H.dev2cell[j]];
        ++j;
      }
      T.c1 = j;
      T.nslots = len;
      const HdrLayout L = hdr_layout(T.c1 - T.c0, F, T.nslots);
      if (L.bytes > kHdrCap - kStageHdrOff) return bfail(b, SGPU_BAD_GRID, "tile header of %d bytes", L.bytes);
      T.hdr = (int)hacc;
      T.hdr_bytes = L.bytes;
      hacc += L.bytes;
      H.tiles.push_back(T);
      acc += (len + 3) & ~3;
    }
  }
  H.n3c = acc;
  for (int j = cd[1]; j < Nc; ++j) {
    H.coff[j] = (int)acc;
    acc += g->Nk[H.dev2cell[j]];
  }
  H.coff[Nc] = (int)acc;
  H.n3 = acc;
  H.ncomp = cd[1];
  H.h_bytes = hacc;
  std::vector<long long> eoff(Ne + 1, 0);
  for (int e = 0; e < Ne; ++e) eoff[e + 1] = eoff[e] + g->Nke[e];
  H.ne3 = eoff[Ne];
  // reserve device ranges (+4 slots: the coefficient stream of a tile reads one group past it)
  H.s_off = b->slots.alloc(H.n3 + 4);
  H.c_off = b->cols.alloc(H.ncomp);
  H.e_off = b->eslots.alloc(std::max(1LL, H.ne3));
  H.h_off = b->hdrs.alloc(H.h_bytes);
  long long ntl = 0;
  for (int i = 0; i < b->max_inst; ++i)
    if (b->inst[i].live) ntl += (long long)b->inst[i].tiles.size();
  if (H.s_off < 0 || H.c_off < 0 || H.e_off < 0 || H.h_off < 0 || ntl + (long long)H.tiles.size() > b->max_tiles) {
    if (H.s_off >= 0) b->slots.release(H.s_off, H.n3 + 4);
    if (H.c_off >= 0) b->cols.release(H.c_off, H.ncomp);
    if (H.e_off >= 0) b->eslots.release(H.e_off, std::max(1LL, H.ne3));
    if (H.h_off >= 0) b->hdrs.release(H.h_off, H.h_bytes);
    return bfail(b, SGPU_OOM, "batch capacity exhausted (slots %lld free of %lld)", b->slots.free_total(),
                 b->max_slots);
  }
  // stage host data (pageable copies; the upload is synchronous per instance)
  Guard gd(b->device);
  std::vector<double> v_dzz(H.n3, 1.0), v_src(H.n3, 0.0), v_q(H.n3, 0.0), v_c(H.n3, 1.0),
      v_dzfD(std::max(1LL, H.ne3));
  for (int j = 0; j < Nc; ++j) {
    const int i = H.dev2cell[j];
    std::memcpy(&v_dzz[H.coff[j]], dzz[i], sizeof(double) * g->Nk[i]);
    std::memcpy(&v_src[H.coff[j]], src[i], sizeof(double) * g->Nk[i]);
    std::memcpy(&v_q[H.coff[j]], q[i], sizeof(double) * g->Nk[i]);
    if (c) std::memcpy(&v_c[H.coff[j]], c[i], sizeof(double) * g->Nk[i]);
  }
  for (int e = 0; e < Ne; ++e)
    for (int k = 0; k < g->Nke[e]; ++k) v_dzfD[eoff[e] + k] = dzf[e][k] * D[e];
  std::vector<BCol> v_col(H.ncomp);
  std::vector<BFace> v_face((size_t)H.ncomp * F);
  std::vector<double> v_Ac(H.ncomp);
  for (int j = 0; j < cd[1]; ++j) {
    const int i = H.dev2cell[j];
    v_col[j].s = (int)(H.s_off + H.coff[j]);
    v_col[j].nk = g->Nk[i];
    v_col[j].ctop = ctop[i];
    v_col[j].inst = id;
    v_Ac[j] = g->Ac[i];
    for (int f = 0; f < F; ++f) {
      BFace& fc = v_face[(size_t)j * F + f];
      fc.ns = -1;
      fc.es = 0;
      fc.kmin = fc.kmax = 0;
      fc.D = 0.f;
      fc.D64 = 0.0;
      if (f >= g->nfaces[i]) continue;
      const int nc = g->neigh[i * F + f], e = g->face[i * F + f];
      if (nc < 0) continue;
      if (e < 0 || e >= Ne || nc >= Nc) return bfail(b, SGPU_BAD_GRID, "face/neigh out of range at cell %d", i);
      if (g->Nke[e] > g->Nk[i] || g->Nke[e] > g->Nk[nc]) return bfail(b, SGPU_BAD_GRID, "Nke exceeds Nk at edge %d", e);
      fc.ns = (int)(H.s_off + H.coff[c2d[nc]]);
      fc.es = (int)(H.e_off + eoff[e]);
      fc.kmin = (short)std::max(ctop[i], ctop[nc]);
      fc.kmax = (short)g->Nke[e];
      fc.D = (float)D[e];
      fc.D64 = D[e];
    }
  }
  // tile headers
  std::vector<unsigned char> v_hdr(std::max(16LL, H.h_bytes), 0);
  for (const HostTile& T : H.tiles) {
    const int ncols = T.c1 - T.c0;
    const HdrLayout L = hdr_layout(ncols, F, T.nslots);
    unsigned char* h = v_hdr.data() + T.hdr;
    int* h0 = (int*)h;
    h0[0] = ncols;
    h0[1] = T.nslots;
    h0[2] = (int)(H.s_off + T.base);
    h0[3] = id;
    unsigned short* st = (unsigned short*)(h + L.o_start);
    int* cn = (int*)(h + L.o_cn);
    int* fns = (int*)(h + L.o_fns);
    int* fkk = (int*)(h + L.o_fkk);
    unsigned char* cmap = h + L.o_cmap;
    for (int cc = 0; cc < ncols; ++cc) {
      const int j = T.c0 + cc;
      st[cc] = (unsigned short)(H.coff[j] - T.base);
      for (int u = H.coff[j] - T.base; u < H.coff[j] - T.base + g->Nk[H.dev2cell[j]]; ++u) cmap[u] = (unsigned char)cc;
      cn[cc] = v_col[j].ctop | (v_col[j].nk << 16);
      for (int f = 0; f < F; ++f) {
        const BFace& fc = v_face[(size_t)j * F + f];
        fns[cc * F + f] = fc.ns;
        fkk[cc * F + f] = fc.ns < 0 ? 0 : ((int)fc.kmin | ((int)fc.kmax << 16));
      }
    }
    st[ncols] = (unsigned short)T.nslots;
  }
  std::vector<float> v_dzfD32(v_dzfD.size());
  for (size_t k = 0; k < v_dzfD.size(); ++k) v_dzfD32[k] = (float)v_dzfD[k];
  cudaStream_t s = b->ustream;
  BCK(cudaMemcpyAsync(b->d_dzz64 + H.s_off, v_dzz.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_src64 + H.s_off, v_src.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_q64 + H.s_off, v_q.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_cin64 + H.s_off, v_c.data(), 8 * H.n3, cudaMemcpyHostToDevice, s));
  if (H.ne3 > 0) {
    BCK(cudaMemcpyAsync(b->d_dzfD64 + H.e_off, v_dzfD.data(), 8 * H.ne3, cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(b->a.dzfD32 + H.e_off, v_dzfD32.data(), 4 * H.ne3, cudaMemcpyHostToDevice, s));
  }
  BCK(cudaMemcpyAsync(b->d_col + H.c_off, v_col.data(), sizeof(BCol) * H.ncomp, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_face + H.c_off * F, v_face.data(), sizeof(BFace) * H.ncomp * F, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_colAc + H.c_off, v_Ac.data(), 8 * H.ncomp, cudaMemcpyHostToDevice, s));
  BCK(cudaMemcpyAsync(b->d_hdrs + H.h_off, v_hdr.data(), H.h_bytes, cudaMemcpyHostToDevice, s));
  // padding slots of the instance must be finite in every FP32 stream (they are copied, never used)
  float* f32s[] = {b->a.fz32, b->a.cinv32, b->a.coef32, b->a.r32, b->a.pa32, b->a.pb32, b->a.x32, b->a.z32};
  for (float* p : f32s) BCK(cudaMemsetAsync(p + H.s_off, 0, 4 * (H.n3 + 4), s));
  if (b->qprecond == 2) BCK(cudaMemsetAsync(b->a.s32 + H.s_off, 0, 4 * (H.n3 + 4), s));
  for (int f = 0; f < F; ++f)
    BCK(cudaMemsetAsync(b->a.fw32 + (size_t)f * b->a.fw_stride + H.s_off, 0, 4 * (H.n3 + 4), s));
  BCK(cudaStreamSynchronize(s));
  BInst& I = b->h_inst[id];
  std::memset(&I, 0, sizeof(BInst));
  I.s0 = (int)(H.s_off);
  I.s1 = (int)(H.s_off + H.n3c);
  I.s2 = (int)(H.s_off + H.n3);
  I.maxiters = qmaxiters;
  I.qprecond = b->qprecond;
  I.tol2 = qepsilon * qepsilon;
  I.resnorm = resnorm;
  I.state = INST_SETUP;
  I.status = SGPU_OK;
  for (int j = 0; j < cd[1]; ++j) H.unk += g->Nk[H.dev2cell[j]] - ctop[H.dev2cell[j]];
  b->inst[id] = std::move(H);
  *id_out = id;
  return SGPU_OK;
}

// Runs up to max_iters global iterations (<= 0: until every instance is done).
// Returns the number of instances still running in *running.
int sgpu_batch_run(sgpu_batch* b, int max_iters, int* running, double* ms, long long* unknown_iters) {
  int rc = sgpu_batch_launch(b, max_iters);
  if (rc != SGPU_OK) return rc;
  return sgpu_batch_wait(b, running, ms, unknown_iters);
}

// Enqueues one launch over every problem in set-up or running state and
// returns at once.  Until sgpu_batch_wait, problems may be added, finished
// problems re-submitted or read back (those touch only problems the launch
// does not run); they join the next launch.
int sgpu_batch_launch(sgpu_batch* b, int max_iters) {
  if (!b) return SGPU_BAD_ARG;
  if (b->inflight) return bfail(b, SGPU_BAD_ARG, "a launch is already in flight");
  Guard gd(b->device);
  int ntiles = 0;
  int ninst = 0;
  bool tiles_changed = false;
  // Tile t runs on CTA t mod G, so the tiles of the problems still iterating
  // stay evenly spread over the CTAs as long as they are a prefix of the tile
  // list: problems are laid out longest expected remaining solve first (their
  // last solve's iteration count less the iterations done; problems never
  // solved before count as longest, larger first).  A problem's reductions
  // group its tiles by their index within the problem modulo G, so the order
  // does not change any result.
  std::vector<int> order;
  std::vector<long long> key(b->max_inst, 0);
  for (int i = 0; i < b->max_inst; ++i) {
    HostInst& H = b->inst[i];
    BInst& I = b->h_inst[i];
    if (!H.live) continue;
    ninst = i + 1;
    b->n_before[i] = (I.state == INST_RUN) ? I.n : 0;
    if (I.state != INST_SETUP && I.state != INST_RUN) {
      I.t0 = I.t1 = 0;
      continue;
    }
    key[i] = H.last_iters > 0 ? std::max(1, H.last_iters - (I.state == INST_RUN ? I.n : 0)) : (1LL << 40);
    order.push_back(i);
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    if (key[x] != key[y]) return key[x] > key[y];
    return b->inst[x].unk > b->inst[y].unk;
  });
  int max_hdr = 0, max_slots = 0;
  for (int i : order) {
    HostInst& H = b->inst[i];
    BInst& I = b->h_inst[i];
    if (I.t0 != ntiles) tiles_changed = true;
    I.t0 = ntiles;
    for (const HostTile& T : H.tiles) {
      if (ntiles >= b->max_tiles) return bfail(b, SGPU_OOM, "too many tiles");
      TileDesc& d = b->h_tiles[ntiles];
      const int nb = (int)(H.h_off + T.hdr), base = (int)(H.s_off + T.base);
      if (d.hdr != nb || d.base != base || d.inst != i) tiles_changed = true;
      d.hdr = nb;
      d.hdr_bytes = T.hdr_bytes;
      max_hdr = std::max(max_hdr, T.hdr_bytes);
      max_slots = std::max(max_slots, T.nslots);
      d.base = base;
      d.nslots = T.nslots;
      d.inst = i;
      d.c0 = (int)(H.c_off + T.c0);
      d.c1 = (int)(H.c_off + T.c1);
      d.pad = 0;
      b->h_tinst[ntiles] = i;
      ++ntiles;
    }
    I.t1 = ntiles;
    I.cnt = 0;
  }
  b->launched = order;
  b->launched_ninst = ninst;
  if (ntiles == 0) {
    b->launched.clear();
    b->last_ms = 0;
    b->last_work = 0;
    return SGPU_OK;
  }
  // stages sized to this launch's largest tile header: the streams start
  // right after it (a 1024-slot tile of 40-level columns has a ~3 KB header,
  // far below the 10 KB a tile of 128 shallow columns needs), which leaves
  // room for three CTAs per SM with the apply phase's 4 + F streams
  const int hdr_cap = std::min(kHdrCap, (kStageHdrOff + max_hdr + 127) & ~127);
  const bool one_pass = b->fusion == 2 && b->qprecond != 2;
  const int streams = one_pass ? b->streams + 1 : (b->x_in_apply ? b->streams : std::max(b->streams - 1, 4));
  // streams sized to the launch's largest tile (+1 group of 4: the vertical
  // coefficient stream reads one slot past the tile)
  const int stream_floats = std::min(kStreamFloats, ((max_slots + 3) & ~3) + 4);
  const int stage_bytes =
      std::max(hdr_cap + streams * 4 * stream_floats, (int)((sizeof(TileSmem) + 127) & ~127));
  b->dyn_smem = dyn_smem_bytes_for(stage_bytes);
  int maxg = batch_max_grid(b, one_pass);
  if (maxg <= 0) return bfail(b, SGPU_CUDA_ERROR, "occupancy query failed");
  int grid = b->grid_override > 0 ? std::min(b->grid_override, maxg) : maxg;
  grid = std::max(1, std::min(grid, ntiles));
  if ((ntiles + grid - 1) / grid > kListCap)
    return bfail(b, SGPU_OOM, "%d tiles exceed %d per CTA at %d CTAs", ntiles, kListCap, grid);
  std::memset(b->h_ctl, 0, sizeof(SolveCtl));
  b->h_ctl->timeout_ns = b->timeout_ns;
  int any_run = 0, any_setup = 0;
  for (int i = 0; i < ninst; ++i) {
    if (!b->inst[i].live) continue;
    any_run |= b->h_inst[i].state == INST_RUN;
    any_setup |= b->h_inst[i].state == INST_SETUP;
  }
  b->h_gflags[0] = 0;
  b->h_gflags[1] = any_setup;
  b->h_gflags[2] = 0;
  b->h_gflags[3] = any_run;
  const int chunk = max_iters > 0 ? max_iters : 0x7fffffff;
  const bool key_same = b->g_ntiles == ntiles && b->g_ninst == ninst && b->g_grid == grid && b->g_chunk == chunk &&
                        b->g_stage == stage_bytes && b->g_hdr == hdr_cap && b->g_sfl == stream_floats &&
                        b->g_fusion == b->fusion && b->g_delta == b->delta &&
                        !tiles_changed;
  cudaStream_t st = b->stream;
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_tiles, b->h_tiles, sizeof(TileDesc) * ntiles, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b->d_tile_inst, b->h_tinst, sizeof(int) * ntiles, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b->d_inst, b->h_inst_up, sizeof(BInst) * ninst, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b->d_ctl, b->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(b->d_gflags, b->h_gflags, 4 * sizeof(int), cudaMemcpyHostToDevice, st))) return e;
    BatchArgs a = b->a;
    a.F = b->F;
    a.stage_bytes = stage_bytes;
    a.hdr_cap = hdr_cap;
    a.stream_floats = stream_floats;
    a.x_in_apply = b->x_in_apply;
    a.one_pass = one_pass ? 1 : 0;
    a.ntiles = ntiles;
    a.ninst = ninst;
    a.max_iters_chunk = chunk;
    a.delta2 = b->delta * b->delta;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = b->dyn_smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&a};
    // the instance table and status come back in sgpu_batch_wait, after the
    // stream has drained: a device-to-host copy queued behind the kernel here
    // would hold up the read-backs of finished problems on the other stream
    return cudaLaunchKernelExC(&cfg, kernel_of(b->qprecond, one_pass), args);
  };
  std::memcpy(b->h_inst_up, b->h_inst, sizeof(BInst) * ninst);
  BCK(cudaEventRecord(b->ev0, st));
  bool launched = false;
  if (b->use_graph) {
    if (!(b->gexec && key_same)) {
      if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
      }
      cudaGraph_t gph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = enqueue();
        e = cudaStreamEndCapture(st, &gph);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, gph, 0);
      if (gph) cudaGraphDestroy(gph);
      if (e != cudaSuccess) {
        cudaGetLastError();
        b->gexec = nullptr;
        b->use_graph = false;  // capture not available: launch directly from now on
        b->graph_failed = true;
      } else {
        b->g_ntiles = ntiles;
        b->g_ninst = ninst;
        b->g_grid = grid;
        b->g_chunk = chunk;
        b->g_stage = stage_bytes;
        b->g_hdr = hdr_cap;
        b->g_sfl = stream_floats;
        b->g_fusion = b->fusion;
        b->g_delta = b->delta;
      }
    }
    if (b->gexec) {
      BCK(cudaGraphLaunch(b->gexec, st));
      launched = true;
      ++b->graph_launches;
    }
  }
  if (!launched) BCK(enqueue());
  BCK(cudaEventRecord(b->ev1, st));
  b->inflight = true;
  return SGPU_OK;
}

// Waits for the launch in flight (none: returns the current counts) and takes
// the state of the problems it ran.  *running counts problems in set-up or
// running state afterwards.
int sgpu_batch_wait(sgpu_batch* b, int* running, double* ms, long long* unknown_iters) {
  if (!b) return SGPU_BAD_ARG;
  Guard gd(b->device);
  long long work = 0;
  float fms = 0.f;
  if (b->inflight) {
    b->inflight = false;
    BCK(cudaStreamSynchronize(b->stream));
    cudaEventElapsedTime(&fms, b->ev0, b->ev1);
    BCK(cudaMemcpyAsync(b->h_inst_dev, b->d_inst, sizeof(BInst) * b->launched_ninst, cudaMemcpyDeviceToHost,
                        b->stream));
    BCK(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    b->last_ms = fms;
    for (int i : b->launched) {
      b->h_inst[i] = b->h_inst_dev[i];
      const BInst& I = b->h_inst[i];
      work += b->inst[i].unk * (long long)(I.n - b->n_before[i]);
      if (I.state == INST_DONE && I.n > 0) b->inst[i].last_iters = I.n;
    }
    b->launched.clear();
    if (b->h_ctl->status == SGPU_TIMEOUT)
      return bfail(b, SGPU_TIMEOUT, "device wait timed out (phase %d)", b->h_ctl->phase_err);
  }
  int run = 0;
  for (int i = 0; i < b->max_inst; ++i) {
    if (!b->inst[i].live) continue;
    const BInst& I = b->h_inst[i];
    run += I.state == INST_RUN || I.state == INST_SETUP;
  }
  b->last_work = work;
  if (running) *running = run;
  if (ms) *ms = fms;
  if (unknown_iters) *unknown_iters = work;
  return SGPU_OK;
}

// Copies an instance's result to the caller's jagged q (computational cells,
// levels [ctop, Nk)) and its report; frees the instance when `release` != 0.
int sgpu_batch_result(sgpu_batch* b, int id, double* const* q, sgpu_stats* st, int release) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live) return SGPU_BAD_ARG;
  HostInst& H = b->inst[id];
  const BInst& I = b->h_inst[id];
  if (st) {
    st->status = I.status;
    st->niters = I.n;
    st->eps = I.eps;
    st->eps0 = I.eps0;
    st->ms_solve = b->last_ms;
    st->ms_total = 0;
    st->unknowns = H.unk;
  }
  if (q) {
    if (I.state != INST_DONE) return bfail(b, SGPU_BAD_ARG, "instance %d has not finished", id);
    Guard gd(b->device);
    // x64 (and c64 for qprecond 1) copied once into pinned staging, then
    // unscaled and scattered row by row
    const long long n = H.n3c, need = (b->qprecond == 1 ? 2 : 1) * n;
    if (b->h_stage_n < need) {
      if (b->h_stage) cudaFreeHost(b->h_stage);
      b->h_stage = nullptr;
      BCK(cudaMallocHost((void**)&b->h_stage, sizeof(double) * need));
      b->h_stage_n = need;
    }
    double* x = b->h_stage;
    double* c = b->h_stage + n;
    BCK(cudaMemcpyAsync(x, b->a.x64 + H.s_off, 8 * n, cudaMemcpyDeviceToHost, b->ustream));
    if (b->qprecond == 1) BCK(cudaMemcpyAsync(c, b->a.c64 + H.s_off, 8 * n, cudaMemcpyDeviceToHost, b->ustream));
    BCK(cudaStreamSynchronize(b->ustream));
    const bool scaled = b->qprecond == 1;
    host_split(H.ncomp, 8192, [&](long long jb, long long je) {
      for (long long j = jb; j < je; ++j) {
        const int i = H.dev2cell[j], k0 = H.ctop[i];
        const long long o = H.coff[j];
        if (scaled)
          for (int k = k0; k < H.Nk[i]; ++k) q[i][k] = x[o + k] * c[o + k];  // c64 holds 1/c
        else
          std::memcpy(q[i] + k0, x + o + k0, sizeof(double) * (H.Nk[i] - k0));
      }
    });
  }
  if (release) {
    b->slots.release(H.s_off, H.n3 + 4);
    b->cols.release(H.c_off, H.ncomp);
    b->eslots.release(H.e_off, std::max(1LL, H.ne3));
    b->hdrs.release(H.h_off, H.h_bytes);
    H = HostInst();
    std::memset(&b->h_inst[id], 0, sizeof(BInst));
  }
  return SGPU_OK;
}

// Re-submits a finished instance.  src (jagged rows of Nk[i] doubles, cell
// order) replaces the right-hand side, or NULL keeps the resident one; with
// warm != 0 the last solution becomes the initial guess (as phys->qc is in the
// model), otherwise the originally uploaded initial guess is used again.  The
// grid and coefficients stay resident.
int sgpu_batch_resubmit(sgpu_batch* b, int id, const double* const* src, double qepsilon, int qmaxiters, int warm) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live) return SGPU_BAD_ARG;
  HostInst& H = b->inst[id];
  BInst& I = b->h_inst[id];
  if (I.state != INST_DONE) return bfail(b, SGPU_BAD_ARG, "instance %d is still running", id);
  Guard gd(b->device);
  const int n = (int)H.n3c;
  if (warm) {
    finalize_q_kernel<<<std::max(1, std::min(1024, (n + 255) / 256)), 256, 0, b->ustream>>>(
        b->a.x64, b->a.c64, b->d_q64, (int)H.s_off, n, b->qprecond == 1);
    BCK(cudaGetLastError());
  }
  if (src) {
    if (b->h_stage_n < H.n3c) {
      if (b->h_stage) cudaFreeHost(b->h_stage);
      b->h_stage = nullptr;
      BCK(cudaMallocHost((void**)&b->h_stage, sizeof(double) * H.n3c));
      b->h_stage_n = H.n3c;
    }
    double* stg = b->h_stage;
    host_split(H.ncomp, 8192, [&](long long jb, long long je) {
      // this range's columns and the padding after each (up to the next column)
      for (long long j = jb; j < je; ++j) {
        const int i = H.dev2cell[j];
        const long long o = H.coff[j], end = (j + 1 < H.ncomp) ? H.coff[j + 1] : H.n3c;
        std::memcpy(stg + o, src[i], sizeof(double) * H.Nk[i]);
        std::fill(stg + o + H.Nk[i], stg + end, 0.0);
      }
    });
    BCK(cudaMemcpyAsync(b->d_src64 + H.s_off, b->h_stage, sizeof(double) * n, cudaMemcpyHostToDevice, b->ustream));
  }
  if (warm || src) BCK(cudaStreamSynchronize(b->ustream));
  I.tol2 = qepsilon * qepsilon;
  I.maxiters = qmaxiters;
  I.state = INST_SETUP;
  I.status = SGPU_OK;
  I.n = 0;
  I.flags = 0;
  return SGPU_OK;
}

int sgpu_batch_use_graph(sgpu_batch* b, int on) {
  if (!b) return SGPU_BAD_ARG;
  b->use_graph = on != 0 && !b->graph_failed;
  return b->use_graph ? 1 : 0;
}

long long sgpu_batch_graph_launches(const sgpu_batch* b) { return b ? b->graph_launches : -1; }

int sgpu_batch_state(const sgpu_batch* b, int id) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live) return -1;
  return b->h_inst[id].state;
}

int sgpu_batch_set(sgpu_batch* b, double delta, int grid, long long timeout_ns) {
  if (!b) return SGPU_BAD_ARG;
  if (delta > 0) b->delta = delta;
  if (grid >= 0) b->grid_override = grid;
  if (timeout_ns > 0) b->timeout_ns = timeout_ns;
  return SGPU_OK;
}

int sgpu_batch_set_fusion(sgpu_batch* b, int form) {
  if (!b || form < 0 || form > 2) return SGPU_BAD_ARG;
  if (b->inflight) return bfail(b, SGPU_BAD_ARG, "a launch is in flight");
  // a problem in mid-solve holds state that only its form reads (a deferred
  // solution increment, the one-pass form's pending step and buffer parity):
  // change the form between solves only
  for (int i = 0; i < b->max_inst; ++i)
    if (b->inst[i].live && b->h_inst[i].state == INST_RUN && form != b->fusion)
      return bfail(b, SGPU_BAD_ARG, "problem %d is in mid-solve", i);
  b->fusion = form;
  b->x_in_apply = form >= 1 ? 1 : 0;  // qprecond 2 runs form 2 as form 1
  return SGPU_OK;
}

int sgpu_batch_set_stride(sgpu_batch* b, int id, int stride) {
  if (!b || id < 0 || id >= b->max_inst || !b->inst[id].live || stride < 1 || stride > 64) return SGPU_BAD_ARG;
  if (b->inflight) return bfail(b, SGPU_BAD_ARG, "a launch is in flight");
  b->h_inst[id].stride = stride;  // uploaded with the instance table at the next launch
  return SGPU_OK;
}

int sgpu_batch_set_tile_slots(sgpu_batch* b, int tile_slots) {
  if (!b || tile_slots < 4 || tile_slots > kBTSlots) return SGPU_BAD_ARG;
  b->tile_slots = tile_slots;
  return SGPU_OK;
}

void* sgpu_batch_stream(sgpu_batch* b) { return b ? (void*)b->stream : nullptr; }

int sgpu_batch_phase_times(const sgpu_batch* b, long long* ns8) {
  if (!b || !ns8) return SGPU_BAD_ARG;
  for (int k = 0; k < 8; ++k) ns8[k] = b->h_ctl ? b->h_ctl->phase_ns[k] : 0;
  return SGPU_OK;
}

}  // extern "C"
