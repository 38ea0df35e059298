// sgpu_common.cuh -- device-side building blocks shared by the solver kernels.
//
//  * GridSync: a grid-wide barrier for cooperative (co-resident) launches whose
//    last-arriving CTA runs a "finaliser" (the deterministic reduction of the
//    per-CTA partial sums and the CG scalar recurrences) before it releases the
//    others.  Every wait is bounded by %globaltimer; on time-out the waiter
//    records SGPU_TIMEOUT in the control block and the kernel returns.
//  * Block reductions in FP64 with a fixed combination order, so every run of
//    the same problem on the same launch shape gives the same bits.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define SGPU_OK 0
#define SGPU_MAXITER 1
#define SGPU_BREAKDOWN 2
#define SGPU_TIMEOUT 3
#define SGPU_OOM 4
#define SGPU_BAD_GRID 5
#define SGPU_BAD_ARG 6
#define SGPU_CUDA_ERROR 7
#define SGPU_NO_DEVICE 8

namespace sgpu {

constexpr int kBlock = 256;        // threads per CTA of the solver kernels
constexpr int kTileCap = 512;      // storage slots per tile (2 per thread)
constexpr int kMaxTileCols = kTileCap;  // a tile may hold up to 512 one-level columns

// Control block of one solve, in device memory.  The barrier words live in
// their own 128-byte lines.
struct __align__(128) SolveCtl {
  // barrier
  unsigned int count;
  unsigned int pad0[31];
  unsigned int gen;
  unsigned int pad1[31];
  // scalars published by the finaliser
  double alpha, alpha0, eps, eps0, mu, nu;
  double res_true;        // optional diagnostic
  int n;                  // iterations executed
  int done;               // 1 = leave the loop
  int status;             // SGPU_* code
  int phase_err;          // where a wait gave up
  long long timeout_ns;   // barrier wait bound
  // per-phase device time, filled only in builds with SGPU_PHASE_TIMING
  long long phase_ns[8];  // indexed by (phase id & 7)
  long long last_ts;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_int(const int* p) {
  return *reinterpret_cast<const volatile int*>(p);
}

// Deterministic FP64 block sum (blockDim.x == BS).  All threads get the result.
template <int NV, int BS = kBlock>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* [NV][BS/32] */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = v[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) smem[j * (BS / 32) + wid] = s;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < BS / 32; ++w) s += smem[j * (BS / 32) + w];
    v[j] = s;
  }
  __syncthreads();
}

// Sum of partials[j*stride + b] over b in [0, n) in a fixed order, by one CTA.
template <int NV>
__device__ __forceinline__ void reduce_partials(const double* partials, int stride, int n, double (&out)[NV],
                                                double* smem) {
  double v[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = 0.0;
    for (int b = threadIdx.x; b < n; b += kBlock) s += ((volatile const double*)partials)[j * stride + b];
    v[j] = s;
  }
  block_sum<NV>(v, smem);
#pragma unroll
  for (int j = 0; j < NV; ++j) out[j] = v[j];
}

// Grid barrier with a finaliser run by the last CTA to arrive.
// Returns false if the kernel must stop (time-out or an error status).
template <class Fin>
__device__ __forceinline__ bool grid_sync(SolveCtl* ctl, int phase, Fin&& fin) {
  __shared__ int s_last;
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int my_gen = ld_acquire_u32(&ctl->gen);
    __threadfence();
    unsigned int old = atomicAdd(&ctl->count, 1u);
    s_last = (old == gridDim.x - 1);
    s_ok = 1;
    if (!s_last) {
      const unsigned long long t0 = globaltimer_ns();
      const unsigned long long lim = (unsigned long long)ctl->timeout_ns;
      unsigned int spins = 0;
      while (ld_acquire_u32(&ctl->gen) == my_gen) {
        if (++spins > 64) __nanosleep(64);
        if ((spins & 255u) == 0 && globaltimer_ns() - t0 > lim) {
          atomicCAS(&ctl->status, SGPU_OK, SGPU_TIMEOUT);
          atomicCAS(&ctl->phase_err, 0, phase);
          s_ok = 0;
          break;
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    fin();           // whole CTA; must end with its own __syncthreads
    __syncthreads();
    if (threadIdx.x == 0) {
      ctl->count = 0u;
      __threadfence();
      atomicAdd(&ctl->gen, 1u);
    }
    __syncthreads();
  }
#ifdef SGPU_PHASE_TIMING
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const long long now = (long long)globaltimer_ns();
    if (ctl->last_ts) ctl->phase_ns[phase & 7] += now - ctl->last_ts;
    ctl->last_ts = now;
  }
#endif
  if (!s_ok) return false;
  return ld_volatile_int(&ctl->status) == SGPU_OK || ld_volatile_int(&ctl->status) == SGPU_MAXITER;
}

__device__ __forceinline__ unsigned int ld_relaxed_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Arrive-and-wait grid barrier on a monotonic counter: the k-th barrier of a
// launch (k = 1, 2, ...) returns once all G CTAs have arrived at it, i.e. once
// ctl->count >= k*G.  No CTA runs a finaliser: after the barrier every CTA
// reduces the published per-CTA partials itself (grid_reduce), in the same
// fixed order, so all CTAs hold the same scalars without a second round trip
// through the control block.  ctl->count must be 0 at launch.
// The arrival is a release reduction (no value returned, nothing to wait for);
// the spin uses relaxed loads, which do not invalidate the SM's L1 as an
// acquire load does (an early CTA spinning with acquire loads would keep
// flushing the L1 of the CTAs still working on the same SM), and one acquire
// fence follows the spin.  The wait is bounded by %globaltimer; on time-out
// SGPU_TIMEOUT and the phase are recorded and false is returned.
__device__ __forceinline__ bool grid_wait(SolveCtl* ctl, unsigned int target, int phase) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&ctl->count), "r"(1u) : "memory");
    if (ld_relaxed_u32(&ctl->count) < target) {
      const unsigned long long t0 = globaltimer_ns();
      const unsigned long long lim = (unsigned long long)ctl->timeout_ns;
      unsigned int spins = 0;
      while (ld_relaxed_u32(&ctl->count) < target) {
        if (++spins > 8) __nanosleep(20);
        if ((spins & 255u) == 0 && globaltimer_ns() - t0 > lim) {
          atomicCAS(&ctl->status, SGPU_OK, SGPU_TIMEOUT);
          atomicCAS(&ctl->phase_err, 0, phase);
          s_ok = 0;
          break;
        }
      }
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
  }
  __syncthreads();
#ifdef SGPU_PHASE_TIMING
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const long long now = (long long)globaltimer_ns();
    if (ctl->last_ts) ctl->phase_ns[phase & 7] += now - ctl->last_ts;
    ctl->last_ts = now;
  }
#endif
  return s_ok != 0;
}

// Phase-timing mark (builds with SGPU_PHASE_TIMING only): CTA 0 adds the time
// since its last mark or barrier to phase_ns[slot].
__device__ __forceinline__ void phase_mark(SolveCtl* ctl, int slot) {
#ifdef SGPU_PHASE_TIMING
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const long long now = (long long)globaltimer_ns();
    if (ctl->last_ts) ctl->phase_ns[slot & 7] += now - ctl->last_ts;
    ctl->last_ts = now;
  }
#endif
}

// FP64 reductions with few FP64 instructions.  GB300 executes about two FP64
// operations per SM and cycle, so a shuffle tree in every warp followed by
// every thread summing the warp results (block_sum) can cost more FP64 issue
// slots than the CG arithmetic it serves.  cta_sum stages the values in shared
// memory and lets one warp add them: BS + 5*32 FP64 additions per value per
// CTA instead of (5 + BS/32)*BS.  The order is fixed, so every run and every
// CTA gives the same bits.  smem holds NV*BS + NV doubles.
template <int NV, int BS>
__device__ __forceinline__ void cta_sum(double (&v)[NV], double* smem) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int j = 0; j < NV; ++j) smem[j * BS + tid] = v[j];
  __syncthreads();
  if (tid < 32) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < BS / 32; ++w) s += smem[j * BS + w * 32 + tid];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (tid == 0) smem[NV * BS + j] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = smem[NV * BS + j];
  __syncthreads();
}

// Sum over b in [0, G) of part[j*G + b] for j < NV, by one warp, read past L1
// (the partials are rewritten by other CTAs between barriers), in the same
// fixed order in every CTA, so every CTA gets the same bits.  Thread 0 then
// runs fin(totals) -- the scalar recurrences, whose results it leaves in
// shared memory for the CTA -- before the closing __syncthreads.
template <int NV, class Fin>
__device__ __forceinline__ void grid_sum(const double* part, int G, Fin&& fin) {
  const int tid = threadIdx.x;
  if (tid < 32) {
    double tot[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int b = tid; b < G; b += 32) s += __ldcg(part + (size_t)j * G + b);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      tot[j] = s;
    }
    if (tid == 0) fin((const double*)tot);
  }
  __syncthreads();
}

}  // namespace sgpu
