// sgpu_noalloc.cu -- the free-surface solve (CGSolve) for callers that cannot
// allocate device memory.
//
// Who needs it: a host program whose device memory is owned entirely by its
// own pool allocator (for example SUNTANS embedded in a coupled model whose
// framework hands every component slices of one arena and forbids other
// allocations), or a time-critical loop that must not pay for cudaMalloc /
// cudaFree, which synchronise the whole device.  Such a caller passes device
// buffers it already owns for the grid, the inputs and the output; this file
// allocates nothing.  The solver's own scratch (coefficients, CG vectors,
// reduction partials, barrier words) lives in one file-scope static __device__
// array of fixed size, which every GPU that loads the library holds until the
// process exits.
//
// Limits and sharing rules (also in include/suntans_gb300.h):
//   * scratch bytes = 512 + 16*kNoallocMaxCtas + 8*Nc*(5 + maxfaces) must fit in
//     kNoallocScratchBytes (32 MiB): about 466,000 quadrilateral cells or
//     524,000 triangles.  Larger grids are rejected with SGPU_TOO_LARGE before
//     any device work.
//   * every call shares the one array and leaves its contents behind; the
//     barrier/control words are cleared at the start of each call.  Two calls
//     whose kernels overlap on the GPU (different streams, or different host
//     threads) race on the array and give wrong answers.
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture.  The address is kept per device and CUDA
//     context: a call after cudaDeviceReset (a new context) looks it up again.
//
// Semantics are those of CGSolve (main/phys.c:3086-3217), HCoefficients
// (3252-3269), OperatorH (3335-3349) and HPreconditioner (3227-3235), with the
// cells visited through cellp in the caller's cell order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>

#include <cuda.h>

#include "../../include/suntans_gb300.h"
#include "sgpu_common.cuh"

namespace sgpu {

constexpr size_t kNoallocScratchBytes = size_t(32) << 20;
constexpr int kNoallocMaxCtas = 2048;
constexpr size_t kCtlBytes = 512;
static_assert(sizeof(SolveCtl) <= kCtlBytes, "control block must fit its slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct NAArgs {
  int Nc, F, ncomp, maxiters, hprecond;
  double epsilon, resnorm, tmp;
  const int* cellp;
  const int* nfaces;
  const int* neigh;
  const int* face;
  const double* Ac;
  const double* df;
  const double* dg;
  const double* D;
  const double* b;   // htmp
  double* x;         // h, in place
  // scratch carved from g_noalloc_scratch
  SolveCtl* ctl;
  double* partials;  // [2*kNoallocMaxCtas]
  double* p;
  double* r;
  double* z;
  double* rt;
  double* hcoef;
  double* hf;        // [Nc*F]
};

static size_t noalloc_bytes(long long Nc, int F) {
  return kCtlBytes + sizeof(double) * 2 * (size_t)kNoallocMaxCtas + sizeof(double) * (size_t)Nc * (5 + F);
}

__global__ void noalloc_init(SolveCtl* ctl, long long timeout_ns) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    unsigned char* c = reinterpret_cast<unsigned char*>(ctl);
    for (size_t i = 0; i < sizeof(SolveCtl); ++i) c[i] = 0;
    ctl->timeout_ns = timeout_ns;
  }
}

__device__ __forceinline__ double na_apply(const NAArgs& a, const double* xin, int i) {
  double y = a.hcoef[i] * xin[i];
  const int nf = a.nfaces[i];
  for (int f = 0; f < nf; ++f) {
    const int nb = a.neigh[i * a.F + f];
    if (nb != -1) y -= a.hf[i * a.F + f] * xin[nb];
  }
  return y;
}

__global__ void __launch_bounds__(kBlock) cgsolve_noalloc_kernel(NAArgs a) {
  __shared__ double s_red[4 * (kBlock / 32)];
  SolveCtl* ctl = a.ctl;
  const int G = gridDim.x, tid = threadIdx.x;
  const int stride = G * kBlock, gid = blockIdx.x * kBlock + tid;

  // coefficients; p = b everywhere except type-3 cells handled below; x = 0 inside
  for (int t = gid; t < a.ncomp; t += stride) {
    const int i = a.cellp[t];
    double cf = a.Ac[i];
    for (int f = 0; f < a.nfaces[i]; ++f) {
      const int nb = a.neigh[i * a.F + f];
      if (nb != -1) {
        const int e = a.face[i * a.F + f];
        const double fc = a.tmp * a.D[e] * a.df[e] / a.dg[e];
        a.hf[i * a.F + f] = fc;
        cf += fc;
      }
    }
    a.hcoef[i] = cf;
    a.x[i] = 0.0;
  }
  // p must read 0 at every non-computational cell (type-3 cells, 3129-3134)
  for (int i = gid; i < a.Nc; i += stride) {
    a.p[i] = 0.0;
    a.z[i] = 0.0;
    a.r[i] = 0.0;
    a.rt[i] = 0.0;
  }
  if (!grid_sync(ctl, 1, [] {})) return;

  {
    double part[2] = {0.0, 0.0};
    for (int t = gid; t < a.ncomp; t += stride) {
      const int i = a.cellp[t];
      const double zi = na_apply(a, a.x, i);
      const double pi = a.b[i] - zi;
      a.r[i] = pi;
      if (a.hprecond == 1) {
        const double rti = pi / a.hcoef[i];
        a.rt[i] = rti;
        a.p[i] = rti;
        part[0] += pi * rti;
        part[1] += pi * pi;
      } else {
        a.p[i] = pi;
        part[0] += pi * pi;
      }
    }
    block_sum<2>(part, s_red);
    if (tid == 0) {
      a.partials[blockIdx.x] = part[0];
      a.partials[kNoallocMaxCtas + blockIdx.x] = part[1];
    }
    if (!grid_sync(ctl, 2, [&] {
          double tot[2];
          reduce_partials<2>(a.partials, kNoallocMaxCtas, G, tot, s_red);
          if (tid == 0) {
            double alpha = tot[0], alpha0 = tot[0];
            if (!a.resnorm) alpha0 = 1;
            const double eps0 = (a.hprecond == 1) ? tot[1] : alpha0;
            ctl->alpha = alpha;
            ctl->alpha0 = alpha0;
            ctl->eps = eps0;
            ctl->eps0 = eps0;
            ctl->n = 0;
            ctl->done = (a.maxiters <= 0 || eps0 == 0 || alpha == 0) ? 1 : 0;
            __threadfence();
          }
        }))
      return;
  }

  for (;;) {
    if (ld_volatile_int(&ctl->done)) break;
    {
      double part[1] = {0.0};
      for (int t = gid; t < a.ncomp; t += stride) {
        const int i = a.cellp[t];
        const double zi = na_apply(a, a.p, i);
        a.z[i] = zi;
        part[0] += a.p[i] * zi;
      }
      block_sum<1>(part, s_red);
      if (tid == 0) a.partials[blockIdx.x] = part[0];
      if (!grid_sync(ctl, 3, [&] {
            double tot[1];
            reduce_partials<1>(a.partials, kNoallocMaxCtas, G, tot, s_red);
            if (tid == 0) {
              const double alpha = *(volatile double*)&ctl->alpha;
              ctl->mu = 1 / alpha;
              const double nu = alpha / tot[0];
              ctl->nu = nu;
              if (!isfinite(nu)) {
                ctl->status = SGPU_BREAKDOWN;
                ctl->done = 1;
              }
              __threadfence();
            }
          }))
        return;
      if (ld_volatile_int(&ctl->done)) break;
    }
    {
      const double nu = *(volatile double*)&ctl->nu;
      double part[2] = {0.0, 0.0};
      for (int t = gid; t < a.ncomp; t += stride) {
        const int i = a.cellp[t];
        a.x[i] += nu * a.p[i];
        const double ri = a.r[i] - nu * a.z[i];
        a.r[i] = ri;
        if (a.hprecond == 1) {
          const double rti = ri / a.hcoef[i];
          a.rt[i] = rti;
          part[0] += ri * rti;
          part[1] += ri * ri;
        } else {
          part[0] += ri * ri;
        }
      }
      block_sum<2>(part, s_red);
      if (tid == 0) {
        a.partials[blockIdx.x] = part[0];
        a.partials[kNoallocMaxCtas + blockIdx.x] = part[1];
      }
      if (!grid_sync(ctl, 4, [&] {
            double tot[2];
            reduce_partials<2>(a.partials, kNoallocMaxCtas, G, tot, s_red);
            if (tid == 0) {
              const double alpha = tot[0];
              double mu = *(volatile double*)&ctl->mu;
              mu *= alpha;
              ctl->mu = mu;
              ctl->alpha = alpha;
              const double eps = (a.hprecond == 1) ? tot[1] : alpha;
              ctl->eps = eps;
              const int n = ctl->n + 1;
              ctl->n = n;
              const bool conv = sqrt(eps / ctl->eps0) < a.epsilon;
              int done = (conv || n >= a.maxiters || eps == 0 || alpha == 0) ? 1 : 0;
              if (!isfinite(alpha)) {
                ctl->status = SGPU_BREAKDOWN;
                done = 1;
              }
              if (done && !conv && n >= a.maxiters && ctl->status == SGPU_OK) ctl->status = SGPU_MAXITER;
              ctl->done = done;
              __threadfence();
            }
          }))
        return;
      if (ld_volatile_int(&ctl->done)) break;
    }
    {
      const double mu = *(volatile double*)&ctl->mu;
      const double* src = (a.hprecond == 1) ? a.rt : a.r;
      for (int t = gid; t < a.ncomp; t += stride) {
        const int i = a.cellp[t];
        a.p[i] = src[i] + mu * a.p[i];
      }
      if (!grid_sync(ctl, 5, [] {})) return;
    }
  }
}

// Device address of g_noalloc_scratch, looked up once per device and context.
// The address belongs to the module loaded into one CUDA context: after
// cudaDeviceReset (or any other end of the device's primary context) the array
// is loaded again at a new address.  So the cached address is keyed by the
// context's unique id (cuCtxGetId, never reused within a process), reached
// through the runtime's driver entry points so that the library needs no link
// against the driver library.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

static std::mutex g_na_mutex;
static void* g_na_ptr[64];
static unsigned long long g_na_ctx[64];
static bool g_na_done[64];
static PfnCtxGetCurrent g_ctx_get_current = nullptr;
static PfnCtxGetId g_ctx_get_id = nullptr;

// id of the context current on this thread; 0 on failure
static unsigned long long current_context_id() {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      return 0;
    g_ctx_get_current = (PfnCtxGetCurrent)f1;
    g_ctx_get_id = (PfnCtxGetId)f2;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS || c == nullptr) return 0;
  if (g_ctx_get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static int noalloc_scratch_ptr(int dev, void** out) {
  if (dev < 0 || dev >= 64) return SGPU_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  unsigned long long id = current_context_id();
  if (!g_na_done[dev] || id == 0 || id != g_na_ctx[dev]) {
    // set-up: the first call on this device (and again after its context changed)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) return SGPU_CUDA_ERROR;
    if (id == 0) id = current_context_id();  // the lookup above made the primary context current
    g_na_ptr[dev] = p;
    g_na_ctx[dev] = id;
    g_na_done[dev] = (id != 0);
  }
  *out = g_na_ptr[dev];
  return SGPU_OK;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" int sgpu_cgsolve_noalloc(const sgpu_noalloc_grid* g, const double* D, double* h, const double* htmp,
                                    const sgpu_props* prop, sgpu_stats* st, void* stream) {
  auto t0 = std::chrono::steady_clock::now();
  if (!g || !D || !h || !htmp || !prop) return SGPU_BAD_ARG;
  if (g->Nc <= 0 || g->maxfaces <= 0 || g->ncomp < 0 || g->ncomp > g->Nc || !g->cellp || !g->nfaces ||
      !g->neigh || !g->face || !g->Ac || !g->df || !g->dg)
    return SGPU_BAD_ARG;
  if (noalloc_bytes(g->Nc, g->maxfaces) > kNoallocScratchBytes) return SGPU_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SGPU_NO_DEVICE;
  void* base = nullptr;
  int rc = noalloc_scratch_ptr(dev, &base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;

  unsigned char* cur = (unsigned char*)base;
  NAArgs a;
  a.ctl = (SolveCtl*)cur;
  cur += kCtlBytes;
  a.partials = (double*)cur;
  cur += sizeof(double) * 2 * (size_t)kNoallocMaxCtas;
  double* v = (double*)cur;
  const size_t Nc = (size_t)g->Nc;
  a.p = v;
  a.r = v + Nc;
  a.z = v + 2 * Nc;
  a.rt = v + 3 * Nc;
  a.hcoef = v + 4 * Nc;
  a.hf = v + 5 * Nc;
  a.Nc = g->Nc;
  a.F = g->maxfaces;
  a.ncomp = g->ncomp;
  a.maxiters = prop->maxiters;
  a.hprecond = prop->hprecond;
  a.epsilon = prop->epsilon;
  a.resnorm = prop->resnorm;
  a.tmp = prop->grav * std::pow(prop->theta * prop->dt, 2);
  a.cellp = g->cellp;
  a.nfaces = g->nfaces;
  a.neigh = g->neigh;
  a.face = g->face;
  a.Ac = g->Ac;
  a.df = g->df;
  a.dg = g->dg;
  a.D = D;
  a.b = htmp;
  a.x = h;

  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return SGPU_CUDA_ERROR;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)cgsolve_noalloc_kernel, kBlock, 0) !=
      cudaSuccess)
    return SGPU_CUDA_ERROR;
  int grid = sms * per;
  grid = std::min(grid, kNoallocMaxCtas);
  grid = std::max(1, std::min(grid, (g->Nc + kBlock - 1) / kBlock));

  noalloc_init<<<1, 1, 0, s>>>(a.ctl, 2000000000LL);
  if (cudaGetLastError() != cudaSuccess) return SGPU_CUDA_ERROR;
  void* args[] = {(void*)&a};
  if (cudaLaunchCooperativeKernel((const void*)cgsolve_noalloc_kernel, dim3(grid), dim3(kBlock), args, 0, s) !=
      cudaSuccess)
    return SGPU_CUDA_ERROR;
  SolveCtl hc;
  if (cudaMemcpyAsync(&hc, a.ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SGPU_CUDA_ERROR;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SGPU_CUDA_ERROR;
  if (st) {
    st->status = hc.status;
    st->niters = hc.n;
    st->eps = hc.eps;
    st->eps0 = hc.eps0;
    st->ms_solve = -1.0;
    st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    st->unknowns = g->ncomp;
  }
  return hc.status;
}
