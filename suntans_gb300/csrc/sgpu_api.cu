// sgpu_api.cu -- the C ABI (include/suntans_gb300.h): grid contexts, host <->
// HBM staging of the reference's jagged arrays, and the solve launches.
//
// Host staging: the jagged rows of q, src, c, dzz (cell order) are gathered
// into pinned buffers in device column order (computational cells in cellp
// order, then type-3 cells, then the rest) with several host threads, then
// copied with one cudaMemcpyAsync per array on the context's stream.  The
// solution is copied back the same way and scattered into the caller's rows for
// computational cells and levels k in [ctop, Nk) only.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/suntans_gb300.h"
#include "sgpu_common.cuh"
#include "sgpu_q.h"
#include "sgpu_step.h"

using namespace sgpu;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct sgpu_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  long long timeout_ns = 2000000000LL;
  int grid_override = 0;

  // host copies of the static grid
  int Nc = 0, Ne = 0, F = 0, Nkmax = 0, ncomp = 0, nbdy = 0;
  std::vector<int> Nk, Nke, nfaces, dev2cell, cell2dev, dcoff, eoff, tile_col, nbr, fedge, slotcol;
  long long n3 = 0, n3c = 0, ne3 = 0;
  int ntiles = 0;

  // device memory (static grid)
  std::vector<void*> allocs;
  int *d_dcoff = nullptr, *d_tile = nullptr, *d_slotcol = nullptr, *d_nk = nullptr, *d_nbr = nullptr, *d_fedge = nullptr,
      *d_nke = nullptr, *d_eoff = nullptr;
  double *d_Ac = nullptr, *d_df = nullptr, *d_dg = nullptr;

  // pressure solve buffers
  bool q_ready = false;
  int *d_ctop = nullptr, *d_fmeta = nullptr, *d_fnoff = nullptr, *d_nslot = nullptr;
  unsigned char* d_sflag = nullptr;
  double *d_dzz = nullptr, *d_dzf = nullptr, *d_Dq = nullptr, *d_qin = nullptr, *d_srcin = nullptr,
         *d_cin = nullptr, *d_coef = nullptr, *d_fc = nullptr, *d_c = nullptr, *d_tw = nullptr,
         *d_tib = nullptr, *d_x = nullptr, *d_p = nullptr, *d_r = nullptr, *d_z = nullptr, *d_rt = nullptr;
  std::vector<int> h_ctop;  // last uploaded ctop (cell order), for the download scatter
  bool q_uploaded = false, q_solved = false;

  // pressure-step buffers (ComputeQSource / Corrector)
  bool step_grid = false, step_ready = false;
  int ncedge = 0;
  long long nw3 = 0;
  std::vector<int> woff;
  int *d_nfaces = nullptr, *d_normal = nullptr, *d_grad = nullptr, *d_cedge = nullptr, *d_woff = nullptr,
      *d_etop = nullptr;
  double *d_u = nullptr, *d_ut2 = nullptr, *d_w = nullptr, *d_wt2 = nullptr, *d_qtot = nullptr;
  // vertical-grid refresh buffers (UpdateDZ / SetFluxHeight)
  bool vgrid_ready = false;
  int *d_ctopold = nullptr, *d_etopold = nullptr;
  double *d_dz = nullptr, *d_dv = nullptr, *d_dzbot = nullptr, *d_hv = nullptr, *d_dzzold = nullptr;

  // WPredictor buffers
  bool wp_ready = false;
  int *d_ecsr = nullptr, *d_eside = nullptr;
  double *d_cnw = nullptr, *d_cnw2 = nullptr, *d_wt = nullptr, *d_wcc = nullptr, *d_wface = nullptr;

  // UPredictor buffers
  std::vector<int> cedge_h;  // computational edges (host copy)
  bool up_grid = false, up_ready = false;
  int nb2 = 0, nbnd = 0;
  int *d_b2edge = nullptr, *d_bedge = nullptr, *d_bnfaces = nullptr, *d_bfedge = nullptr, *d_bnormal = nullptr,
      *d_mark = nullptr, *d_nnan = nullptr;
  double *d_n1 = nullptr, *d_n2 = nullptr, *d_utmp = nullptr, *d_E = nullptr, *d_tauT = nullptr, *d_CdT = nullptr,
         *d_CdB = nullptr, *d_nutv = nullptr, *d_nulax = nullptr;
  unsigned char* d_active = nullptr;

  // free-surface buffers
  bool h_ready = false;
  double *d_Dh = nullptr, *d_hin = nullptr, *d_bin = nullptr, *d_hcoef = nullptr, *d_hf = nullptr,
         *d_hx = nullptr, *d_hp = nullptr, *d_hr = nullptr, *d_hz = nullptr, *d_hrt = nullptr,
         *d_hihc = nullptr, *d_hp1 = nullptr;
  int* d_hn = nullptr;
  bool h_uploaded = false, h_solved = false;

  // control
  SolveCtl* d_ctl = nullptr;
  double* d_partials = nullptr;
  int partials_cap = 0;
  SolveCtl* h_ctl = nullptr;  // pinned

  // pinned staging
  double* pin = nullptr;
  size_t pin_elems = 0;
};

static int fail(sgpu_context* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? SGPU_OOM : SGPU_CUDA_ERROR, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                        \
  } while (0)

template <class T>
static int dalloc(sgpu_context* ctx, T** p, size_t n) {
  void* v = nullptr;
  CK(cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T)));
  ctx->allocs.push_back(v);
  *p = (T*)v;
  return SGPU_OK;
}

template <class T>
static int upload(sgpu_context* ctx, T** p, const T* host, size_t n) {
  int rc = dalloc(ctx, p, n);
  if (rc) return rc;
  if (n) CK(cudaMemcpyAsync(*p, host, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return SGPU_OK;
}

static int ensure_pinned(sgpu_context* ctx, size_t elems) {
  if (ctx->pin_elems >= elems) return SGPU_OK;
  if (ctx->pin) {
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->pin);
    ctx->pin = nullptr;
    ctx->pin_elems = 0;
  }
  CK(cudaMallocHost((void**)&ctx->pin, elems * sizeof(double)));
  ctx->pin_elems = elems;
  return SGPU_OK;
}

// parallel host loop over [0, n)
template <class Fn>
static void host_parallel(long long n, Fn&& fn) {
  unsigned hw = std::thread::hardware_concurrency();
  int nt = (int)std::min<long long>(std::max(1u, std::min(hw, 16u)), std::max(1LL, n / 65536));
  if (nt <= 1) {
    fn(0LL, n);
    return;
  }
  std::vector<std::thread> th;
  long long chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    long long b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) th.emplace_back([&fn, b, e] { fn(b, e); });
  }
  for (auto& x : th) x.join();
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

extern "C" {

const char* sgpu_status_string(int s) {
  switch (s) {
    case SGPU_OK: return "ok";
    case SGPU_MAXITER: return "maxiter";
    case SGPU_BREAKDOWN: return "breakdown";
    case SGPU_TIMEOUT: return "timeout";
    case SGPU_OOM: return "out of memory";
    case SGPU_BAD_GRID: return "bad grid";
    case SGPU_BAD_ARG: return "bad argument";
    case SGPU_CUDA_ERROR: return "cuda error";
    case SGPU_NO_DEVICE: return "no cuda device";
    case SGPU_TOO_LARGE: return "grid exceeds the fixed scratch of the allocation-free solve";
  }
  return "unknown";
}

const char* sgpu_last_error(const sgpu_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sgpu_destroy(sgpu_context* ctx) {
  if (!ctx) return SGPU_BAD_ARG;
  {
    DeviceGuard g(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (void* p : ctx->allocs) cudaFree(p);
    if (ctx->pin) cudaFreeHost(ctx->pin);
    if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
  return SGPU_OK;
}

static int build_layout(sgpu_context* ctx, const sgpu_grid_desc* g) {
  const int Nc = g->Nc, Ne = g->Ne, mf = g->maxfaces;
  if (Nc <= 0 || Ne < 0 || mf <= 0 || g->Nkmax <= 0) return fail(ctx, SGPU_BAD_GRID, "empty or negative sizes");
  if (!g->nfaces || !g->neigh || !g->face || !g->Nk || !g->Nke || !g->cellp || !g->celldist || !g->Ac || !g->df ||
      !g->dg)
    return fail(ctx, SGPU_BAD_ARG, "null array in grid description");
  const int* cd = g->celldist;
  if (!(cd[0] == 0 && cd[0] <= cd[1] && cd[1] <= cd[2] && cd[2] <= Nc))
    return fail(ctx, SGPU_BAD_GRID, "celldist must satisfy 0 = c0 <= c1 <= c2 <= Nc");
  if (g->Nkmax > kTileCap) return fail(ctx, SGPU_BAD_GRID, "Nkmax %d exceeds %d", g->Nkmax, kTileCap);
  ctx->Nc = Nc;
  ctx->Ne = Ne;
  ctx->F = mf;
  ctx->Nkmax = g->Nkmax;
  ctx->ncomp = cd[1];
  ctx->nbdy = cd[2] - cd[1];
  ctx->Nk.assign(g->Nk, g->Nk + Nc);
  ctx->Nke.assign(g->Nke, g->Nke + Ne);
  ctx->nfaces.assign(g->nfaces, g->nfaces + Nc);
  for (int i = 0; i < Nc; ++i) {
    if (g->Nk[i] < 1 || g->Nk[i] > g->Nkmax) return fail(ctx, SGPU_BAD_GRID, "Nk[%d]=%d out of [1,Nkmax]", i, g->Nk[i]);
    if (g->nfaces[i] < 1 || g->nfaces[i] > mf)
      return fail(ctx, SGPU_BAD_GRID, "nfaces[%d]=%d out of [1,maxfaces]", i, g->nfaces[i]);
  }
  // device order
  ctx->cell2dev.assign(Nc, -1);
  ctx->dev2cell.clear();
  ctx->dev2cell.reserve(Nc);
  for (int t = 0; t < cd[2]; ++t) {
    const int i = g->cellp[t];
    if (i < 0 || i >= Nc || ctx->cell2dev[i] >= 0) return fail(ctx, SGPU_BAD_GRID, "cellp[%d]=%d invalid or repeated", t, i);
    ctx->cell2dev[i] = (int)ctx->dev2cell.size();
    ctx->dev2cell.push_back(i);
  }
  for (int i = 0; i < Nc; ++i)
    if (ctx->cell2dev[i] < 0) {
      ctx->cell2dev[i] = (int)ctx->dev2cell.size();
      ctx->dev2cell.push_back(i);
    }
  ctx->dcoff.assign(Nc + 1, 0);
  long long acc = 0;
  for (int j = 0; j < Nc; ++j) {
    ctx->dcoff[j] = (int)acc;
    acc += g->Nk[ctx->dev2cell[j]];
    if (acc > 0x7fffff00LL) return fail(ctx, SGPU_BAD_GRID, "more than 2^31 storage slots");
  }
  ctx->dcoff[Nc] = (int)acc;
  ctx->n3 = acc;
  ctx->n3c = ctx->dcoff[ctx->ncomp];
  ctx->eoff.assign(Ne + 1, 0);
  acc = 0;
  for (int e = 0; e < Ne; ++e) {
    ctx->eoff[e] = (int)acc;
    acc += g->Nke[e];
  }
  ctx->eoff[Ne] = (int)acc;
  ctx->ne3 = acc;
  if (acc > 0x7fffff00LL) return fail(ctx, SGPU_BAD_GRID, "more than 2^31 edge slots");
  // neighbours of computational columns
  const int ncomp = ctx->ncomp;
  ctx->nbr.assign((size_t)std::max(ncomp, 1) * mf, -1);
  ctx->fedge.assign((size_t)std::max(ncomp, 1) * mf, 0);
  for (int j = 0; j < ncomp; ++j) {
    const int i = ctx->dev2cell[j];
    for (int f = 0; f < g->nfaces[i]; ++f) {
      const int nc = g->neigh[i * mf + f], e = g->face[i * mf + f];
      if (e < 0 || e >= Ne) return fail(ctx, SGPU_BAD_GRID, "face[%d]=%d out of range", i * mf + f, e);
      ctx->fedge[(size_t)j * mf + f] = e;
      if (nc < -1 || nc >= Nc) return fail(ctx, SGPU_BAD_GRID, "neigh[%d]=%d out of range", i * mf + f, nc);
      if (nc >= 0) {
        if (g->Nke[e] > g->Nk[i] || g->Nke[e] > g->Nk[nc])
          return fail(ctx, SGPU_BAD_GRID, "Nke[%d]=%d exceeds Nk of cell %d or %d", e, g->Nke[e], i, nc);
        ctx->nbr[(size_t)j * mf + f] = ctx->cell2dev[nc];
      }
    }
  }
  // tiles of whole computational columns, <= kTileCap slots each
  ctx->tile_col.clear();
  ctx->tile_col.push_back(0);
  int cur = 0;
  for (int j = 0; j < ncomp; ++j) {
    const int len = g->Nk[ctx->dev2cell[j]];
    if (cur + len > kTileCap) {
      ctx->tile_col.push_back(j);
      cur = 0;
    }
    cur += len;
  }
  if (ncomp > 0) ctx->tile_col.push_back(ncomp);
  ctx->ntiles = (int)ctx->tile_col.size() - 1;
  ctx->slotcol.assign((size_t)std::max(1, ctx->dcoff[ncomp]), 0);
  for (int j = 0; j < ncomp; ++j)
    for (int u = ctx->dcoff[j]; u < ctx->dcoff[j + 1]; ++u) ctx->slotcol[u] = j;
  return SGPU_OK;
}

int sgpu_create(const sgpu_grid_desc* g, int device, sgpu_context** out) {
  if (!g || !out) return SGPU_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return SGPU_NO_DEVICE;
  if (device < 0 || device >= ndev) return SGPU_BAD_ARG;
  sgpu_context* ctx = new sgpu_context();
  ctx->device = device;
  int rc = build_layout(ctx, g);
  if (rc) {
    // keep the message reachable through a context with no device memory
    *out = ctx;
    return rc;
  }
  DeviceGuard dg(device);
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  CK(cudaMallocHost((void**)&ctx->h_ctl, sizeof(SolveCtl)));
  std::vector<double> Acd(ctx->Nc);
  for (int j = 0; j < ctx->Nc; ++j) Acd[j] = g->Ac[ctx->dev2cell[j]];
  std::vector<int> nkd(ctx->Nc);
  for (int j = 0; j < ctx->Nc; ++j) nkd[j] = g->Nk[ctx->dev2cell[j]];
  if ((rc = upload(ctx, &ctx->d_dcoff, ctx->dcoff.data(), ctx->dcoff.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_tile, ctx->tile_col.data(), ctx->tile_col.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_slotcol, ctx->slotcol.data(), ctx->slotcol.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_nk, nkd.data(), nkd.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_nbr, ctx->nbr.data(), ctx->nbr.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_fedge, ctx->fedge.data(), ctx->fedge.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_nke, ctx->Nke.data(), ctx->Nke.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_eoff, ctx->eoff.data(), ctx->eoff.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_Ac, Acd.data(), Acd.size()))) return rc;
  if ((rc = upload(ctx, &ctx->d_df, g->df, (size_t)ctx->Ne))) return rc;
  if ((rc = upload(ctx, &ctx->d_dg, g->dg, (size_t)ctx->Ne))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_ctl, 1))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  *out = ctx;
  return SGPU_OK;
}

int sgpu_set_timeout_ns(sgpu_context* ctx, long long ns) {
  if (!ctx || ns <= 0) return SGPU_BAD_ARG;
  ctx->timeout_ns = ns;
  return SGPU_OK;
}

int sgpu_set_grid(sgpu_context* ctx, int ctas) {
  if (!ctx || ctas < 0) return SGPU_BAD_ARG;
  ctx->grid_override = ctas;
  return SGPU_OK;
}

void* sgpu_stream(sgpu_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int sgpu_phase_times(const sgpu_context* ctx, long long* ns8) {
  if (!ctx || !ns8) return SGPU_BAD_ARG;
  for (int k = 0; k < 8; ++k) ns8[k] = ctx->h_ctl ? ctx->h_ctl->phase_ns[k] : 0;
  return SGPU_OK;
}

static int ensure_partials(sgpu_context* ctx, int grid) {
  if (ctx->partials_cap >= grid) return SGPU_OK;
  int rc = dalloc(ctx, &ctx->d_partials, (size_t)8 * grid);  // up to 8 doubles per CTA (free surface: 6)
  if (rc) return rc;
  ctx->partials_cap = grid;
  return SGPU_OK;
}

static int alloc_q(sgpu_context* ctx) {
  if (ctx->q_ready) return SGPU_OK;
  const size_t n3 = ctx->n3 + 1, n3c = ctx->n3c + 1, ncf = (size_t)std::max(ctx->ncomp, 1) * ctx->F;
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_ctop, ctx->Nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_fmeta, ncf))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_fnoff, ncf))) return rc;
  double** v[] = {&ctx->d_dzz, &ctx->d_qin, &ctx->d_srcin, &ctx->d_cin, &ctx->d_coef, &ctx->d_c,
                  &ctx->d_x,   &ctx->d_p,   &ctx->d_r,     &ctx->d_z,   &ctx->d_rt};
  for (auto pp : v)
    if ((rc = dalloc(ctx, pp, n3))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_tw, n3c))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_tib, n3c))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_fc, n3c * ctx->F))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_nslot, n3c * ctx->F))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_sflag, n3c))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dzf, ctx->ne3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_Dq, ctx->Ne + 1))) return rc;
  CK(cudaMemsetAsync(ctx->d_coef, 0, n3 * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_tw, 0, n3c * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_tib, 0, n3c * sizeof(double), ctx->stream));
  ctx->q_ready = true;
  return SGPU_OK;
}

// gather jagged rows (cell order) into pinned staging in device column order
static void gather_cells(sgpu_context* ctx, const double* const* rows, double* dst) {
  host_parallel(ctx->Nc, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j];
      std::memcpy(dst + ctx->dcoff[j], rows[i], sizeof(double) * ctx->Nk[i]);
    }
  });
}

int sgpu_q_upload(sgpu_context* ctx, const int* ctop, const double* const* dzz, const double* const* dzf,
                  const double* D, const double* const* q, const double* const* src, const double* const* c) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctop || !dzz || !dzf || !D || !q || !src) return fail(ctx, SGPU_BAD_ARG, "null argument");
  DeviceGuard dg(ctx->device);
  int rc = alloc_q(ctx);
  if (rc) return rc;
  const size_t n3 = ctx->n3, ne3 = ctx->ne3;
  for (int i = 0; i < ctx->Nc; ++i)
    if (ctop[i] < 0 || ctop[i] >= ctx->Nk[i]) return fail(ctx, SGPU_BAD_ARG, "ctop[%d]=%d out of [0,Nk)", i, ctop[i]);
  // staging: [ctop as int | dzz | q | src | c | dzf | D]
  const size_t n_ctop = (ctx->Nc + 1) / 2 + 1;
  const size_t need = n_ctop + 4 * n3 + ne3 + ctx->Ne + 8;
  if ((rc = ensure_pinned(ctx, need))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));  // staging reuse
  int* s_ctop = (int*)ctx->pin;
  double* s_dzz = ctx->pin + n_ctop;
  double* s_q = s_dzz + n3;
  double* s_src = s_q + n3;
  double* s_c = s_src + n3;
  double* s_dzf = s_c + n3;
  double* s_D = s_dzf + ne3;
  // each array goes up as soon as it is gathered, so its copy overlaps the next gather
  cudaStream_t st = ctx->stream;
  for (int j = 0; j < ctx->Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  ctx->h_ctop.assign(ctop, ctop + ctx->Nc);
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * ctx->Nc, cudaMemcpyHostToDevice, st));
  gather_cells(ctx, dzz, s_dzz);
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  gather_cells(ctx, q, s_q);
  CK(cudaMemcpyAsync(ctx->d_qin, s_q, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  gather_cells(ctx, src, s_src);
  CK(cudaMemcpyAsync(ctx->d_srcin, s_src, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  // c is read only at the type-3 boundary columns (the solver conditions the
  // computational ones itself), so only their slots go up
  const size_t n3c = ctx->n3c;
  if (n3 > n3c) {
    for (int j = ctx->ncomp; j < ctx->Nc; ++j) {
      const int i = ctx->dev2cell[j];
      if (c) std::memcpy(s_c + ctx->dcoff[j], c[i], sizeof(double) * ctx->Nk[i]);
      else std::fill(s_c + ctx->dcoff[j], s_c + ctx->dcoff[j] + ctx->Nk[i], 1.0);
    }
    CK(cudaMemcpyAsync(ctx->d_cin + n3c, s_c + n3c, sizeof(double) * (n3 - n3c), cudaMemcpyHostToDevice, st));
  }
  host_parallel(ctx->Ne, [&](long long b, long long e) {
    for (long long k = b; k < e; ++k) std::memcpy(s_dzf + ctx->eoff[k], dzf[k], sizeof(double) * ctx->Nke[k]);
  });
  CK(cudaMemcpyAsync(ctx->d_dzf, s_dzf, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  std::memcpy(s_D, D, sizeof(double) * ctx->Ne);
  CK(cudaMemcpyAsync(ctx->d_Dq, s_D, sizeof(double) * ctx->Ne, cudaMemcpyHostToDevice, st));
  ctx->q_uploaded = true;
  ctx->q_solved = false;
  return SGPU_OK;
}

static void reset_ctl(sgpu_context* ctx) {
  std::memset(ctx->h_ctl, 0, sizeof(SolveCtl));
  ctx->h_ctl->timeout_ns = ctx->timeout_ns;
}

static int run_solve_common(sgpu_context* ctx, sgpu_stats* st, long long unknowns, int grid,
                            cudaError_t (*launch)(sgpu_context*, int, void*), void* arg) {
  reset_ctl(ctx);
  CK(cudaMemcpyAsync(ctx->d_ctl, ctx->h_ctl, sizeof(SolveCtl), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  cudaError_t le = launch(ctx, grid, arg);
  if (le != cudaSuccess)
    return fail(ctx, SGPU_CUDA_ERROR, "solver launch failed: %s", cudaGetErrorString(le));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  const SolveCtl& h = *ctx->h_ctl;
  if (st) {
    st->status = h.status;
    st->niters = h.n;
    st->eps = h.eps;
    st->eps0 = h.eps0;
    st->ms_solve = ms;
    st->unknowns = unknowns;
  }
  if (h.status == SGPU_TIMEOUT) return fail(ctx, SGPU_TIMEOUT, "device barrier wait timed out in phase %d", h.phase_err);
  return h.status;
}

struct QLaunch {
  QArgs a;
  int qprecond;
};

static cudaError_t launch_q_cb2(sgpu_context* ctx, int grid, void* arg) {
  QLaunch* L = (QLaunch*)arg;
  return q_launch(L->a, L->qprecond, grid, ctx->stream);
}

int sgpu_q_solve(sgpu_context* ctx, const sgpu_props* prop, sgpu_stats* st) {
  if (!ctx || !prop) return SGPU_BAD_ARG;
  if (!ctx->q_uploaded) return fail(ctx, SGPU_BAD_ARG, "sgpu_q_solve before sgpu_q_upload");
  if (prop->qprecond < 0 || prop->qprecond > 2) return fail(ctx, SGPU_BAD_ARG, "qprecond must be 0, 1 or 2");
  auto t0 = std::chrono::steady_clock::now();
  DeviceGuard dg(ctx->device);
  int maxg = q_max_grid(prop->qprecond, ctx->device);
  if (maxg <= 0) return fail(ctx, SGPU_CUDA_ERROR, "occupancy query failed");
  // a full wave for large problems; small ones (a few hundred thousand
  // unknowns) take fewer CTAs -- at least one per SM, at least 8 slots per
  // thread -- since their iterations are bound by the grid barriers, whose
  // cost grows with the CTAs arriving
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const long long want = (ctx->n3c + 8LL * kBlock - 1) / (8LL * kBlock);
  int grid = ctx->grid_override > 0 ? std::min(ctx->grid_override, maxg)
                                    : (int)std::min<long long>(maxg, std::max<long long>(sms, want));
  int rc = ensure_partials(ctx, grid);
  if (rc) return rc;
  QLaunch L;
  QArgs& a = L.a;
  a.F = ctx->F;
  a.ncomp = ctx->ncomp;
  a.ncols = ctx->Nc;
  a.n3c = (int)ctx->n3c;
  a.n3 = (int)ctx->n3;
  a.ntiles = ctx->ntiles;
  a.maxiters = prop->qmaxiters;
  a.qepsilon = prop->qepsilon;
  a.resnorm = prop->resnorm;
  a.dcoff = ctx->d_dcoff;
  a.tile_col = ctx->d_tile;
  a.slotcol = ctx->d_slotcol;
  a.nk = ctx->d_nk;
  a.nbr = ctx->d_nbr;
  a.fedge = ctx->d_fedge;
  a.nke = ctx->d_nke;
  a.eoff = ctx->d_eoff;
  a.Ac = ctx->d_Ac;
  a.ctop = ctx->d_ctop;
  a.dzz = ctx->d_dzz;
  a.dzf = ctx->d_dzf;
  a.D = ctx->d_Dq;
  a.q_in = ctx->d_qin;
  a.src_in = ctx->d_srcin;
  a.c_in = ctx->d_cin;
  a.fmeta = ctx->d_fmeta;
  a.fnoff = ctx->d_fnoff;
  a.coef = ctx->d_coef;
  a.fc = ctx->d_fc;
  a.nslot = ctx->d_nslot;
  a.sflag = ctx->d_sflag;
  a.c = ctx->d_c;
  a.tw = ctx->d_tw;
  a.tib = ctx->d_tib;
  a.x = ctx->d_x;
  a.p = ctx->d_p;
  a.r = ctx->d_r;
  a.z = ctx->d_z;
  a.rt = ctx->d_rt;
  a.ctl = ctx->d_ctl;
  a.partials = ctx->d_partials;
  L.qprecond = prop->qprecond;
  long long unk = 0;
  for (int j = 0; j < ctx->ncomp; ++j) unk += ctx->Nk[ctx->dev2cell[j]] - ctx->h_ctop[ctx->dev2cell[j]];
  rc = run_solve_common(ctx, st, unk, grid, launch_q_cb2, &L);
  if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (rc == SGPU_OK || rc == SGPU_MAXITER || rc == SGPU_BREAKDOWN) ctx->q_solved = true;
  return rc;
}

int sgpu_q_download(sgpu_context* ctx, double* const* q) {
  if (!ctx || !q) return SGPU_BAD_ARG;
  if (!ctx->q_solved) return fail(ctx, SGPU_BAD_ARG, "sgpu_q_download before a solve");
  DeviceGuard dg(ctx->device);
  int rc = ensure_pinned(ctx, ctx->n3c + 1);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->pin, ctx->d_x, sizeof(double) * ctx->n3c, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const double* s = ctx->pin;
  host_parallel(ctx->ncomp, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j];
      const int k0 = ctx->h_ctop[i];
      std::memcpy(q[i] + k0, s + ctx->dcoff[j] + k0, sizeof(double) * (ctx->Nk[i] - k0));
    }
  });
  return SGPU_OK;
}

int sgpu_cgsolveq(sgpu_context* ctx, const int* ctop, const double* const* dzz, const double* const* dzf,
                  const double* D, double* const* q, const double* const* src, const double* const* c,
                  const sgpu_props* prop, sgpu_stats* st) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = sgpu_q_upload(ctx, ctop, dzz, dzf, D, (const double* const*)q, src, c);
  if (rc) return rc;
  int src_rc = sgpu_q_solve(ctx, prop, st);
  if (src_rc != SGPU_OK && src_rc != SGPU_MAXITER && src_rc != SGPU_BREAKDOWN) return src_rc;
  rc = sgpu_q_download(ctx, q);
  if (rc) return rc;
  if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return src_rc;
}

// ---------------------------------------------------------------------------
// free surface
// ---------------------------------------------------------------------------
static int alloc_h(sgpu_context* ctx) {
  if (ctx->h_ready) return SGPU_OK;
  const size_t nc = ctx->Nc + 1, ncf = (size_t)std::max(ctx->ncomp, 1) * ctx->F;
  int rc;
  double** v[] = {&ctx->d_hin, &ctx->d_bin, &ctx->d_hcoef, &ctx->d_hx, &ctx->d_hp, &ctx->d_hr, &ctx->d_hz, &ctx->d_hrt,
                  &ctx->d_hihc, &ctx->d_hp1};
  for (auto pp : v)
    if ((rc = dalloc(ctx, pp, nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_hf, ncf))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_hn, ncf))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_Dh, ctx->Ne + 1))) return rc;
  ctx->h_ready = true;
  return SGPU_OK;
}

int sgpu_h_upload(sgpu_context* ctx, const double* D, const double* h, const double* htmp) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!D || !h || !htmp) return fail(ctx, SGPU_BAD_ARG, "null argument");
  DeviceGuard dg(ctx->device);
  int rc = alloc_h(ctx);
  if (rc) return rc;
  if ((rc = ensure_pinned(ctx, 2 * (size_t)ctx->Nc + ctx->Ne + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  double* s_h = ctx->pin;
  double* s_b = s_h + ctx->Nc;
  double* s_D = s_b + ctx->Nc;
  for (int j = 0; j < ctx->Nc; ++j) {
    s_h[j] = h[ctx->dev2cell[j]];
    s_b[j] = htmp[ctx->dev2cell[j]];
  }
  std::memcpy(s_D, D, sizeof(double) * ctx->Ne);
  CK(cudaMemcpyAsync(ctx->d_hin, s_h, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_bin, s_b, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_Dh, s_D, sizeof(double) * ctx->Ne, cudaMemcpyHostToDevice, ctx->stream));
  ctx->h_uploaded = true;
  ctx->h_solved = false;
  return SGPU_OK;
}

struct HLaunch {
  HArgs a;
};

static cudaError_t launch_h_cb(sgpu_context* ctx, int grid, void* arg) {
  return h_launch(((HLaunch*)arg)->a, grid, ctx->stream);
}

int sgpu_h_solve(sgpu_context* ctx, const sgpu_props* prop, sgpu_stats* st) {
  if (!ctx || !prop) return SGPU_BAD_ARG;
  if (!ctx->h_uploaded) return fail(ctx, SGPU_BAD_ARG, "sgpu_h_solve before sgpu_h_upload");
  auto t0 = std::chrono::steady_clock::now();
  DeviceGuard dg(ctx->device);
  int maxg = h_max_grid(ctx->device);
  if (maxg <= 0) return fail(ctx, SGPU_CUDA_ERROR, "occupancy query failed");
  // default: one CTA per SM (the barrier's cost grows with the CTAs arriving)
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  int grid = ctx->grid_override > 0 ? std::min(ctx->grid_override, maxg) : std::min(std::max(sms, 1), maxg);
  // no more CTAs than needed to give every thread a cell
  grid = std::max(1, std::min(grid, (ctx->ncomp + h_block() - 1) / h_block()));
  int rc = ensure_partials(ctx, grid);
  if (rc) return rc;
  HLaunch L;
  HArgs& a = L.a;
  a.F = ctx->F;
  a.ncomp = ctx->ncomp;
  a.ncells = ctx->Nc;
  a.maxiters = prop->maxiters;
  a.hprecond = prop->hprecond;
  a.epsilon = prop->epsilon;
  a.resnorm = prop->resnorm;
  a.tmp = prop->grav * std::pow(prop->theta * prop->dt, 2);
  a.cpc = std::max(1, (ctx->ncomp + grid - 1) / grid);
  a.nbr = ctx->d_nbr;
  a.fedge = ctx->d_fedge;
  a.Ac = ctx->d_Ac;
  a.df = ctx->d_df;
  a.dg = ctx->d_dg;
  a.D = ctx->d_Dh;
  a.h_in = ctx->d_hin;
  a.b_in = ctx->d_bin;
  a.hcoef = ctx->d_hcoef;
  a.ihcoef = ctx->d_hihc;
  a.hf = ctx->d_hf;
  a.hn = ctx->d_hn;
  a.x = ctx->d_hx;
  a.p = ctx->d_hp;
  a.p1 = ctx->d_hp1;
  a.r = ctx->d_hr;
  a.z = ctx->d_hz;
  a.rt = ctx->d_hrt;
  a.ctl = ctx->d_ctl;
  a.partials = ctx->d_partials;
  rc = run_solve_common(ctx, st, ctx->ncomp, grid, launch_h_cb, &L);
  if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (rc == SGPU_OK || rc == SGPU_MAXITER || rc == SGPU_BREAKDOWN) ctx->h_solved = true;
  return rc;
}

int sgpu_h_download(sgpu_context* ctx, double* h) {
  if (!ctx || !h) return SGPU_BAD_ARG;
  if (!ctx->h_solved) return fail(ctx, SGPU_BAD_ARG, "sgpu_h_download before a solve");
  DeviceGuard dg(ctx->device);
  int rc = ensure_pinned(ctx, ctx->Nc + 1);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->pin, ctx->d_hx, sizeof(double) * ctx->ncomp, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int j = 0; j < ctx->ncomp; ++j) h[ctx->dev2cell[j]] = ctx->pin[j];
  return SGPU_OK;
}

int sgpu_cgsolve(sgpu_context* ctx, const double* D, double* h, const double* htmp, const sgpu_props* prop,
                 sgpu_stats* st) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = sgpu_h_upload(ctx, D, h, htmp);
  if (rc) return rc;
  int s_rc = sgpu_h_solve(ctx, prop, st);
  if (s_rc != SGPU_OK && s_rc != SGPU_MAXITER && s_rc != SGPU_BREAKDOWN) return s_rc;
  rc = sgpu_h_download(ctx, h);
  if (rc) return rc;
  if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return s_rc;
}



// ---------------------------------------------------------------------------
// the steps around CGSolveQ: ComputeQSource, Corrector, and the fused step
// ---------------------------------------------------------------------------
static int alloc_step(sgpu_context* ctx) {
  if (ctx->step_ready) return SGPU_OK;
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_u, ctx->ne3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_ut2, ctx->ne3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_w, (size_t)ctx->nw3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_wt2, (size_t)ctx->nw3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_qtot, ctx->n3 + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_etop, (size_t)ctx->Ne + 1))) return rc;
  ctx->step_ready = true;
  return SGPU_OK;
}

int sgpu_step_grid(sgpu_context* ctx, const int* normal, const int* grad, const int* edgep, const int* edgedist) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!normal || !grad || !edgedist || (!edgep && edgedist[1] > edgedist[0])) return fail(ctx, SGPU_BAD_ARG, "null argument");
  const int Nc = ctx->Nc, Ne = ctx->Ne, F = ctx->F, ncomp = ctx->ncomp;
  if (edgedist[0] < 0 || edgedist[1] < edgedist[0]) return fail(ctx, SGPU_BAD_GRID, "edgedist out of order");
  std::vector<int> nf(std::max(ncomp, 1)), nrm((size_t)std::max(ncomp, 1) * F, 0), gd(2 * (size_t)std::max(Ne, 1), -1),
      ce;
  for (int j = 0; j < ncomp; ++j) {
    const int i = ctx->dev2cell[j];
    nf[j] = ctx->nfaces[i];
    for (int f = 0; f < nf[j]; ++f) {
      const int v = normal[(size_t)i * F + f];
      if (v != 1 && v != -1) return fail(ctx, SGPU_BAD_GRID, "normal[%d]=%d is not +1 or -1", i * F + f, v);
      nrm[(size_t)j * F + f] = v;
    }
  }
  for (int e = 0; e < Ne; ++e)
    for (int s = 0; s < 2; ++s) {
      const int c = grad[2 * e + s];
      if (c < -1 || c >= Nc) return fail(ctx, SGPU_BAD_GRID, "grad[%d]=%d out of range", 2 * e + s, c);
      gd[2 * (size_t)e + s] = c < 0 ? -1 : ctx->cell2dev[c];
    }
  for (int t = edgedist[0]; t < edgedist[1]; ++t) {
    const int e = edgep[t];
    if (e < 0 || e >= Ne) return fail(ctx, SGPU_BAD_GRID, "edgep[%d]=%d out of range", t, e);
    if (gd[2 * (size_t)e] < 0 || gd[2 * (size_t)e + 1] < 0)
      return fail(ctx, SGPU_BAD_GRID, "computational edge %d lacks a cell on one side", e);
    ce.push_back(e);
  }
  // each computational column's computational edges, in the caller's edge order (WPredictor adds their
  // horizontal-diffusion terms in that order): 2*edge + side, side 0 where the column is grad[0]
  std::vector<int> ecsr(std::max(ncomp, 0) + 1, 0), eside;
  {
    std::vector<std::vector<int>> per(std::max(ncomp, 0));
    for (int e : ce)
      for (int sd = 0; sd < 2; ++sd) {
        const int c = gd[2 * (size_t)e + sd];
        if (c >= 0 && c < ncomp) per[c].push_back(2 * e + sd);
      }
    for (int j = 0; j < ncomp; ++j) {
      ecsr[j + 1] = ecsr[j] + (int)per[j].size();
      eside.insert(eside.end(), per[j].begin(), per[j].end());
    }
  }
  // deepest edges first: the per-edge kernels (UPredictor's vertical solve, Corrector) stride over this list,
  // so each thread gets a like share of levels and the lanes of a warp have like column lengths
  std::stable_sort(ce.begin(), ce.end(), [&](int x, int y) { return ctx->Nke[x] > ctx->Nke[y]; });
  ctx->woff.assign(Nc + 1, 0);
  for (int j = 0; j < Nc; ++j) ctx->woff[j + 1] = ctx->woff[j] + ctx->Nk[ctx->dev2cell[j]] + 1;
  ctx->nw3 = ctx->woff[Nc];
  DeviceGuard dg(ctx->device);
  int rc;
  if (!ctx->step_grid) {
    if ((rc = dalloc(ctx, &ctx->d_nfaces, nf.size()))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_normal, nrm.size()))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_grad, gd.size()))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_woff, ctx->woff.size()))) return rc;
    if ((rc = dalloc(ctx, &ctx->d_cedge, (size_t)std::max(Ne, 1)))) return rc;
  }
  CK(cudaMemcpyAsync(ctx->d_nfaces, nf.data(), sizeof(int) * nf.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_normal, nrm.data(), sizeof(int) * nrm.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_grad, gd.data(), sizeof(int) * gd.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_woff, ctx->woff.data(), sizeof(int) * ctx->woff.size(), cudaMemcpyHostToDevice,
                     ctx->stream));
  if (!ce.empty())
    CK(cudaMemcpyAsync(ctx->d_cedge, ce.data(), sizeof(int) * ce.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!ctx->d_ecsr && (rc = dalloc(ctx, &ctx->d_ecsr, (size_t)std::max(ncomp, 0) + 1))) return rc;
  if (!ctx->d_eside && (rc = dalloc(ctx, &ctx->d_eside, 2 * (size_t)std::max(Ne, 1)))) return rc;
  CK(cudaMemcpyAsync(ctx->d_ecsr, ecsr.data(), sizeof(int) * ecsr.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!eside.empty())
    CK(cudaMemcpyAsync(ctx->d_eside, eside.data(), sizeof(int) * eside.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->ncedge = (int)ce.size();
  ctx->cedge_h = ce;
  ctx->step_grid = true;
  return SGPU_OK;
}

static StepArgs step_args(sgpu_context* ctx, double theta, double dt) {
  StepArgs a{};
  a.n3 = (int)ctx->n3;
  a.n3c = (int)ctx->n3c;
  a.ncomp = ctx->ncomp;
  a.Ne = ctx->Ne;
  a.F = ctx->F;
  a.ncedge = ctx->ncedge;
  a.thetafactor = (1 - theta) / theta;
  a.dt = dt;
  a.dcoff = ctx->d_dcoff;
  a.woff = ctx->d_woff;
  a.slotcol = ctx->d_slotcol;
  a.nk = ctx->d_nk;
  a.nfaces = ctx->d_nfaces;
  a.fedge = ctx->d_fedge;
  a.normal = ctx->d_normal;
  a.nke = ctx->d_nke;
  a.eoff = ctx->d_eoff;
  a.grad = ctx->d_grad;
  a.cedge = ctx->d_cedge;
  a.Ac = ctx->d_Ac;
  a.df = ctx->d_df;
  a.dg = ctx->d_dg;
  a.ctop = ctx->d_ctop;
  a.etop = ctx->d_etop;
  a.dzz = ctx->d_dzz;
  a.dzf = ctx->d_dzf;
  a.u = ctx->d_u;
  a.utmp2 = ctx->d_ut2;
  a.w = ctx->d_w;
  a.wtmp2 = ctx->d_wt2;
  a.src = ctx->d_srcin;
  a.D = ctx->d_Dq;
  a.u_out = ctx->d_u;
  a.w_out = ctx->d_w;
  a.q_out = ctx->d_qtot;
  return a;
}

static void gather_edges(sgpu_context* ctx, const double* const* rows, double* dst) {
  host_parallel(ctx->Ne, [&](long long b, long long e) {
    for (long long k = b; k < e; ++k) std::memcpy(dst + ctx->eoff[k], rows[k], sizeof(double) * ctx->Nke[k]);
  });
}
static void scatter_edges(sgpu_context* ctx, const double* src, double* const* rows) {
  host_parallel(ctx->Ne, [&](long long b, long long e) {
    for (long long k = b; k < e; ++k) std::memcpy(rows[k], src + ctx->eoff[k], sizeof(double) * ctx->Nke[k]);
  });
}
static void gather_wrows(sgpu_context* ctx, const double* const* rows, double* dst) {
  host_parallel(ctx->Nc, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j];
      std::memcpy(dst + ctx->woff[j], rows[i], sizeof(double) * (ctx->Nk[i] + 1));
    }
  });
}
static void scatter_wrows(sgpu_context* ctx, const double* src, double* const* rows, int ncols) {
  host_parallel(ncols, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j];
      std::memcpy(rows[i], src + ctx->woff[j], sizeof(double) * (ctx->Nk[i] + 1));
    }
  });
}
// cell rows, levels [ctop, Nk) of the first ncols device columns
static void scatter_cells_active(sgpu_context* ctx, const double* src, double* const* rows, const int* ctop,
                                 int ncols) {
  host_parallel(ncols, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j], k0 = ctop[i];
      std::memcpy(rows[i] + k0, src + ctx->dcoff[j] + k0, sizeof(double) * (ctx->Nk[i] - k0));
    }
  });
}

static int check_ctop(sgpu_context* ctx, const int* ctop) {
  for (int i = 0; i < ctx->Nc; ++i)
    if (ctop[i] < 0 || ctop[i] >= ctx->Nk[i]) return fail(ctx, SGPU_BAD_ARG, "ctop[%d]=%d out of [0,Nk)", i, ctop[i]);
  return SGPU_OK;
}

int sgpu_compute_qsource(sgpu_context* ctx, const int* ctop, const double* const* dzf, const double* const* u,
                         const double* const* utmp2, const double* const* w, const double* const* wtmp2,
                         double theta, double dt, double* const* src, double* D) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctop || !dzf || !u || !utmp2 || !w || !wtmp2 || !src || !D) return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  if (!(theta != 0) || !(dt != 0)) return fail(ctx, SGPU_BAD_ARG, "theta and dt must be nonzero");
  int rc;
  if ((rc = check_ctop(ctx, ctop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx))) return rc;
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, nw3 = ctx->nw3, n_ctop = (ctx->Nc + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, n_ctop + 3 * ne3 + 2 * nw3 + n3 + ctx->Ne + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  double* s_dzf = ctx->pin + n_ctop;
  double* s_u = s_dzf + ne3;
  double* s_ut2 = s_u + ne3;
  double* s_w = s_ut2 + ne3;
  double* s_wt2 = s_w + nw3;
  for (int j = 0; j < ctx->Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  gather_edges(ctx, dzf, s_dzf);
  gather_edges(ctx, u, s_u);
  gather_edges(ctx, utmp2, s_ut2);
  gather_wrows(ctx, w, s_w);
  gather_wrows(ctx, wtmp2, s_wt2);
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzf, s_dzf, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_ut2, s_ut2, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_w, s_w, sizeof(double) * nw3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_wt2, s_wt2, sizeof(double) * nw3, cudaMemcpyHostToDevice, ctx->stream));
  StepArgs a = step_args(ctx, theta, dt);
  CK(launch_qsource(a, ctx->stream));
  double* s_src = ctx->pin + n_ctop;  // staging reused after the uploads complete
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpyAsync(s_src, ctx->d_srcin, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(D, ctx->d_Dq, sizeof(double) * ctx->Ne, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  scatter_cells_active(ctx, s_src, src, ctop, ctx->Nc);  // every cell's levels [ctop, Nk), as the reference
  ctx->q_uploaded = false;
  return SGPU_OK;
}

int sgpu_corrector(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                   const double* const* qc, const double* D, double dt, double* const* u, double* const* w,
                   double* const* q) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctop || !etop || !dzz || !qc || !D || !u || !w || !q) return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  int rc;
  if ((rc = check_ctop(ctx, ctop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx))) return rc;
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, nw3 = ctx->nw3, n_ctop = (ctx->Nc + 1) / 2 + 1,
               n_etop = (ctx->Ne + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, n_ctop + n_etop + 3 * n3 + ne3 + nw3 + ctx->Ne + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  int* s_etop = (int*)(ctx->pin + n_ctop);
  double* s_dzz = ctx->pin + n_ctop + n_etop;
  double* s_qc = s_dzz + n3;
  double* s_q = s_qc + n3;
  double* s_u = s_q + n3;
  double* s_w = s_u + ne3;
  double* s_D = s_w + nw3;
  for (int j = 0; j < ctx->Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  for (int e = 0; e < ctx->Ne; ++e) s_etop[e] = etop[e];
  gather_cells(ctx, dzz, s_dzz);
  gather_cells(ctx, qc, s_qc);
  gather_cells(ctx, (const double* const*)q, s_q);
  gather_edges(ctx, (const double* const*)u, s_u);
  gather_wrows(ctx, (const double* const*)w, s_w);
  std::memcpy(s_D, D, sizeof(double) * ctx->Ne);
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * ctx->Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_qin, s_qc, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_qtot, s_q, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_w, s_w, sizeof(double) * nw3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_Dq, s_D, sizeof(double) * ctx->Ne, cudaMemcpyHostToDevice, ctx->stream));
  StepArgs a = step_args(ctx, 1.0, dt);
  a.qc = ctx->d_qin;
  CK(launch_corrector(a, ctx->stream));
  CK(cudaMemcpyAsync(s_u, ctx->d_u, sizeof(double) * ne3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_w, ctx->d_w, sizeof(double) * nw3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_q, ctx->d_qtot, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  scatter_edges(ctx, s_u, u);
  scatter_wrows(ctx, s_w, w, ctx->ncomp);
  scatter_cells_active(ctx, s_q, q, ctop, ctx->ncomp);
  ctx->q_uploaded = false;
  return SGPU_OK;
}

static int alloc_upred(sgpu_context* ctx);
static int alloc_wpred(sgpu_context* ctx);
static int kmax_for(int Nkmax);
static WPredArgs wpred_args(sgpu_context* ctx, const sgpu_wpred_fields* f, const sgpu_props* prop);
static void scatter_cells_all(sgpu_context* ctx, const double* src, double* const* rows);

// ComputeQSource -> CGSolveQ -> Corrector with the right-hand side and the
// correction in HBM; with wf, WPredictor first (its w, the pressure q and the
// histories stay in HBM into ComputeQSource and Corrector).
static int pressure_step_impl(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                              const double* const* dzf, const double* const* utmp2, const double* const* wtmp2,
                              double* const* u, double* const* w, double* const* q, double* const* qc,
                              const double* const* c, const sgpu_wpred_fields* wf, double* const* Cn_W,
                              double* const* Cn_W2, const sgpu_props* prop, sgpu_stats* st) {
  auto t0 = std::chrono::steady_clock::now();
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctop || !etop || !dzz || !dzf || !utmp2 || !wtmp2 || !u || !w || !q || !qc || !prop)
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  if (!(prop->theta != 0) || !(prop->dt != 0)) return fail(ctx, SGPU_BAD_ARG, "theta and dt must be nonzero");
  if (wf) {
    if (!wf->nu_tv || !wf->nu_lax || !Cn_W || !Cn_W2) return fail(ctx, SGPU_BAD_ARG, "null argument");
    if (wf->nonlinear != 0 && wf->nonlinear != 1)
      return fail(ctx, SGPU_BAD_ARG, "WPredictor on the device supports nonlinear 0 and 1, not %d", wf->nonlinear);
    if (wf->conserveMomentum) return fail(ctx, SGPU_BAD_ARG, "WPredictor on the device needs conserveMomentum 0");
    if (ctx->Nkmax + 1 > 128) return fail(ctx, SGPU_BAD_GRID, "WPredictor on the device needs Nkmax <= 127");
    if (ctx->F > 8) return fail(ctx, SGPU_BAD_GRID, "WPredictor on the device needs maxfaces <= 8");
  }
  int rc;
  if ((rc = check_ctop(ctx, ctop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx))) return rc;
  if (wf && ((rc = alloc_upred(ctx)) || (rc = alloc_wpred(ctx)))) return rc;
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, nw3 = ctx->nw3, n_ctop = (ctx->Nc + 1) / 2 + 1,
               n_etop = (ctx->Ne + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, n_ctop + n_etop + (wf ? 8 : 4) * n3 + 3 * ne3 + 2 * nw3 + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  int* s_etop = (int*)(ctx->pin + n_ctop);
  double* s_dzz = ctx->pin + n_ctop + n_etop;
  double* s_qc = s_dzz + n3;
  double* s_q = s_qc + n3;
  double* s_c = s_q + n3;
  double* s_dzf = s_c + n3;
  double* s_u = s_dzf + ne3;
  double* s_ut2 = s_u + ne3;
  double* s_w = s_ut2 + ne3;
  double* s_wt2 = s_w + nw3;
  double* s_nt = s_wt2 + nw3;  // WPredictor only: nu_tv, nu_lax, Cn_W, Cn_W2
  double* s_nl = s_nt + n3;
  double* s_c1 = s_nl + n3;
  double* s_c2 = s_c1 + n3;
  for (int j = 0; j < ctx->Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  for (int e = 0; e < ctx->Ne; ++e) s_etop[e] = etop[e];
  ctx->h_ctop.assign(ctop, ctop + ctx->Nc);
  gather_cells(ctx, dzz, s_dzz);
  gather_cells(ctx, (const double* const*)qc, s_qc);
  gather_cells(ctx, (const double* const*)q, s_q);
  for (int j = ctx->ncomp; j < ctx->Nc; ++j) {  // c is read only at the type-3 boundary columns
    const int i = ctx->dev2cell[j];
    if (c) std::memcpy(s_c + ctx->dcoff[j], c[i], sizeof(double) * ctx->Nk[i]);
    else std::fill(s_c + ctx->dcoff[j], s_c + ctx->dcoff[j] + ctx->Nk[i], 1.0);
  }
  gather_edges(ctx, dzf, s_dzf);
  gather_edges(ctx, (const double* const*)u, s_u);
  gather_edges(ctx, utmp2, s_ut2);
  gather_wrows(ctx, (const double* const*)w, s_w);
  gather_wrows(ctx, wtmp2, s_wt2);
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * ctx->Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_qin, s_qc, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_qtot, s_q, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  if (n3 > (size_t)ctx->n3c)
    CK(cudaMemcpyAsync(ctx->d_cin + ctx->n3c, s_c + ctx->n3c, sizeof(double) * (n3 - ctx->n3c), cudaMemcpyHostToDevice,
                       ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzf, s_dzf, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_ut2, s_ut2, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_w, s_w, sizeof(double) * nw3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_wt2, s_wt2, sizeof(double) * nw3, cudaMemcpyHostToDevice, ctx->stream));
  if (wf) {
    gather_cells(ctx, wf->nu_tv, s_nt);
    gather_cells(ctx, wf->nu_lax, s_nl);
    gather_cells(ctx, (const double* const*)Cn_W, s_c1);
    gather_cells(ctx, (const double* const*)Cn_W2, s_c2);
    CK(cudaMemcpyAsync(ctx->d_nutv, s_nt, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_nulax, s_nl, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_cnw, s_c1, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_cnw2, s_c2, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
    // WPredictor on the uploaded w, u (advecting velocity utmp2) and q
    WPredArgs wa = wpred_args(ctx, wf, prop);
    if (wf->nonlinear) CK(cudaMemsetAsync(ctx->d_wface, 0, sizeof(double) * ne3, ctx->stream));
    CK(launch_wpredictor(wa, ctx->stream));
  }
  // ComputeQSource straight into the solver's right-hand side and D
  StepArgs a = step_args(ctx, prop->theta, prop->dt);
  CK(launch_qsource(a, ctx->stream));
  ctx->q_uploaded = true;
  ctx->q_solved = false;
  rc = sgpu_q_solve(ctx, prop, st);
  if (rc != SGPU_OK && rc != SGPU_MAXITER && rc != SGPU_BREAKDOWN) return rc;
  // Corrector with the solution, still on the device
  a.qc = ctx->d_x;
  CK(launch_corrector(a, ctx->stream));
  CK(cudaMemcpyAsync(s_qc, ctx->d_x, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_q, ctx->d_qtot, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_u, ctx->d_u, sizeof(double) * ne3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_w, ctx->d_w, sizeof(double) * nw3, cudaMemcpyDeviceToHost, ctx->stream));
  if (wf) {
    CK(cudaMemcpyAsync(s_c1, ctx->d_cnw, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(s_c2, ctx->d_cnw2, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  scatter_cells_active(ctx, s_qc, qc, ctop, ctx->ncomp);
  scatter_cells_active(ctx, s_q, q, ctop, ctx->ncomp);
  scatter_edges(ctx, s_u, u);
  scatter_wrows(ctx, s_w, w, ctx->ncomp);
  if (wf) {
    scatter_cells_all(ctx, s_c1, Cn_W);
    scatter_cells_all(ctx, s_c2, Cn_W2);
  }
  if (st) st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int sgpu_pressure_step(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                       const double* const* dzf, const double* const* utmp2, const double* const* wtmp2,
                       double* const* u, double* const* w, double* const* q, double* const* qc,
                       const double* const* c, const sgpu_props* prop, sgpu_stats* st) {
  return pressure_step_impl(ctx, ctop, etop, dzz, dzf, utmp2, wtmp2, u, w, q, qc, c, nullptr, nullptr, nullptr, prop,
                            st);
}

int sgpu_nonhydrostatic_step(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                             const double* const* dzf, const double* const* utmp2, const double* const* wtmp2,
                             const sgpu_wpred_fields* wf, double* const* u, double* const* w, double* const* q,
                             double* const* qc, const double* const* c, double* const* Cn_W, double* const* Cn_W2,
                             const sgpu_props* prop, sgpu_stats* st) {
  if (!wf) return ctx ? fail(ctx, SGPU_BAD_ARG, "null argument") : SGPU_BAD_ARG;
  return pressure_step_impl(ctx, ctop, etop, dzz, dzf, utmp2, wtmp2, u, w, q, qc, c, wf, Cn_W, Cn_W2, prop, st);
}



// ---------------------------------------------------------------------------
// the vertical grid of the step: UpdateDZ (option 0) and SetFluxHeight
// ---------------------------------------------------------------------------
static int alloc_vgrid(sgpu_context* ctx) {
  if (ctx->vgrid_ready) return SGPU_OK;
  int rc;
  if ((rc = dalloc(ctx, &ctx->d_ctopold, ctx->Nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_etopold, (size_t)ctx->Ne + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dz, (size_t)ctx->Nkmax + 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dv, ctx->Nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dzbot, ctx->Nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_hv, ctx->Nc))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dzzold, ctx->n3 + 1))) return rc;
  ctx->vgrid_ready = true;
  return SGPU_OK;
}

static VGridArgs vgrid_args(sgpu_context* ctx, const sgpu_vgrid* v, int linearFS) {
  VGridArgs a{};
  a.Nc = ctx->Nc;
  a.Ne = ctx->Ne;
  a.Nkmax = ctx->Nkmax;
  a.n3 = (int)ctx->n3;
  a.linearFS = linearFS;
  a.smoothbot = v->smoothbot;
  a.dzsmall = v->dzsmall;
  a.dcoff = ctx->d_dcoff;
  a.nk = ctx->d_nk;
  a.nke = ctx->d_nke;
  a.eoff = ctx->d_eoff;
  a.grad = ctx->d_grad;
  a.dz = ctx->d_dz;
  a.dv = ctx->d_dv;
  a.dzbot = ctx->d_dzbot;
  a.h = ctx->d_hv;
  a.u = ctx->d_u;
  a.ctop = ctx->d_ctop;
  a.etop = ctx->d_etop;
  a.ctopold = ctx->d_ctopold;
  a.etopold = ctx->d_etopold;
  a.dzz = ctx->d_dzz;
  a.dzzold = ctx->d_dzzold;
  a.dzf = ctx->d_dzf;
  return a;
}

// the per-cell (device order) and per-level uploads shared by both calls
static int upload_vgrid_common(sgpu_context* ctx, const sgpu_vgrid* v, const double* h, double* s_dv, double* s_dzbot,
                               double* s_h) {
  for (int j = 0; j < ctx->Nc; ++j) {
    const int i = ctx->dev2cell[j];
    s_dv[j] = v->dv[i];
    s_dzbot[j] = v->dzbot ? v->dzbot[i] : 0.0;
    s_h[j] = h[i];
  }
  CK(cudaMemcpyAsync(ctx->d_dz, v->dz, sizeof(double) * ctx->Nkmax, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dv, s_dv, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzbot, s_dzbot, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_hv, s_h, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  return SGPU_OK;
}

static void scatter_cells_all(sgpu_context* ctx, const double* src, double* const* rows) {
  host_parallel(ctx->Nc, [&](long long b, long long e) {
    for (long long j = b; j < e; ++j) {
      const int i = ctx->dev2cell[j];
      std::memcpy(rows[i], src + ctx->dcoff[j], sizeof(double) * ctx->Nk[i]);
    }
  });
}

int sgpu_update_dz(sgpu_context* ctx, const sgpu_vgrid* v, const double* h, int linearFS, int* ctop, int* etop,
                   double* const* dzz, int* ctopold, int* etopold, double* const* dzzold) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!v || !v->dz || !v->dv || !h || !ctop || !etop || !dzz || !ctopold || !etopold || !dzzold)
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  if (linearFS) return SGPU_OK;  // UpdateDZ returns at once for a linearised free surface (822-824)
  int rc;
  if ((rc = check_ctop(ctx, ctop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx)) || (rc = alloc_vgrid(ctx))) return rc;
  const size_t n3 = ctx->n3, Nc = ctx->Nc, Ne = ctx->Ne, ni = (Nc + Ne + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, 2 * ni + 2 * n3 + 3 * Nc + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  int* s_etop = s_ctop + Nc;
  double* s_dzz = ctx->pin + ni;
  double* s_old = s_dzz + n3;
  double* s_dv = s_old + n3;
  double* s_dzbot = s_dv + Nc;
  double* s_h = s_dzbot + Nc;
  for (size_t j = 0; j < Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  std::memcpy(s_etop, etop, sizeof(int) * Ne);
  gather_cells(ctx, (const double* const*)dzz, s_dzz);
  if ((rc = upload_vgrid_common(ctx, v, h, s_dv, s_dzbot, s_h))) return rc;
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * Nc, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  VGridArgs a = vgrid_args(ctx, v, linearFS);
  CK(launch_update_dz(a, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int* o_ctop = (int*)(ctx->pin);
  int* o_etop = o_ctop + Nc;
  CK(cudaMemcpyAsync(o_ctop, ctx->d_ctop, sizeof(int) * Nc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(o_etop, ctx->d_etop, sizeof(int) * Ne, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_dzz, ctx->d_dzz, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_old, ctx->d_dzzold, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<int> old_c(Nc), old_e(Ne + 1);
  CK(cudaMemcpyAsync(old_c.data(), ctx->d_ctopold, sizeof(int) * Nc, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(old_e.data(), ctx->d_etopold, sizeof(int) * Ne, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (size_t j = 0; j < Nc; ++j) {
    const int i = ctx->dev2cell[j];
    ctop[i] = o_ctop[j];
    ctopold[i] = old_c[j];
  }
  std::memcpy(etop, o_etop, sizeof(int) * Ne);
  std::memcpy(etopold, old_e.data(), sizeof(int) * Ne);
  scatter_cells_all(ctx, s_dzz, dzz);
  scatter_cells_all(ctx, s_old, dzzold);
  ctx->q_uploaded = false;
  return SGPU_OK;
}

int sgpu_set_flux_height(sgpu_context* ctx, const sgpu_vgrid* v, const int* etop, const double* h,
                         const double* const* u, double* const* dzz, double* const* dzf) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!v || !v->dz || !v->dv || !v->Nkc || !etop || !h || !u || !dzz || !dzf) return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (v->smoothbot != 0 && !v->dzbot) return fail(ctx, SGPU_BAD_ARG, "dzbot is needed when smoothbot != 0");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  for (int e = 0; e < ctx->Ne; ++e)
    if (v->Nkc[e] < ctx->Nke[e]) return fail(ctx, SGPU_BAD_ARG, "Nkc[%d]=%d below Nke", e, v->Nkc[e]);
  int rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx)) || (rc = alloc_vgrid(ctx))) return rc;
  const size_t n3 = ctx->n3, Nc = ctx->Nc, Ne = ctx->Ne, ne3 = ctx->ne3, ni = (Ne + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, ni + n3 + 2 * ne3 + 3 * Nc + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_etop = (int*)ctx->pin;
  double* s_dzz = ctx->pin + ni;
  double* s_u = s_dzz + n3;
  double* s_dzf = s_u + ne3;
  double* s_dv = s_dzf + ne3;
  double* s_dzbot = s_dv + Nc;
  double* s_h = s_dzbot + Nc;
  std::memcpy(s_etop, etop, sizeof(int) * Ne);
  gather_cells(ctx, (const double* const*)dzz, s_dzz);
  gather_edges(ctx, u, s_u);
  if ((rc = upload_vgrid_common(ctx, v, h, s_dv, s_dzbot, s_h))) return rc;
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, ctx->stream));
  VGridArgs a = vgrid_args(ctx, v, 0);
  CK(launch_set_flux_height(a, ctx->stream));
  CK(cudaMemcpyAsync(s_dzf, ctx->d_dzf, sizeof(double) * ne3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_dzz, ctx->d_dzz, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  host_parallel(ctx->Ne, [&](long long b, long long e) {
    for (long long k = b; k < e; ++k) {
      std::memcpy(dzf[k], s_dzf + ctx->eoff[k], sizeof(double) * ctx->Nke[k]);
      for (int l = ctx->Nke[k]; l < v->Nkc[k]; ++l) dzf[k][l] = 0;  // rows beyond Nke (4380-4383)
    }
  });
  if (v->smoothbot != 0) scatter_cells_all(ctx, s_dzz, dzz);
  ctx->q_uploaded = false;
  return SGPU_OK;
}

// ---------------------------------------------------------------------------
// UPredictor: the predictor around CGSolve
// ---------------------------------------------------------------------------
static int alloc_upred(sgpu_context* ctx) {
  if (ctx->up_ready) return SGPU_OK;
  int rc;
  const size_t ne3 = ctx->ne3 + 1, n3 = ctx->n3 + 1, Ne = ctx->Ne + 1;
  if ((rc = dalloc(ctx, &ctx->d_utmp, ne3)) || (rc = dalloc(ctx, &ctx->d_E, ne3))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_tauT, Ne)) || (rc = dalloc(ctx, &ctx->d_CdT, Ne)) || (rc = dalloc(ctx, &ctx->d_CdB, Ne)))
    return rc;
  if ((rc = dalloc(ctx, &ctx->d_nutv, n3)) || (rc = dalloc(ctx, &ctx->d_nulax, n3))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_active, (size_t)ctx->Nc + 1)) || (rc = dalloc(ctx, &ctx->d_nnan, 1))) return rc;
  ctx->up_ready = true;
  return SGPU_OK;
}

int sgpu_upredictor_grid(sgpu_context* ctx, const int* edgep, const int* edgedist, const int* mark, const double* n1,
                         const double* n2, const int* face, const int* normal) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!edgedist || !mark || !n1 || !n2 || !face || !normal) return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  const int Ne = ctx->Ne, F = ctx->F, nb3 = ctx->nbdy;
  for (int m = 0; m < 5; ++m)
    if (edgedist[m] < 0 || edgedist[m + 1] < edgedist[m] || edgedist[m + 1] > Ne)
      return fail(ctx, SGPU_BAD_GRID, "edgedist out of order");
  if (!edgep && edgedist[5] > 0) return fail(ctx, SGPU_BAD_ARG, "null edgep");
  std::vector<int> b2, bn, bnf(std::max(nb3, 1)), bfe((size_t)std::max(nb3, 1) * F, 0), bnr((size_t)std::max(nb3, 1) * F, 0);
  for (int t = edgedist[2]; t < edgedist[5]; ++t) {
    const int e = edgep[t];
    if (e < 0 || e >= Ne) return fail(ctx, SGPU_BAD_GRID, "edgep[%d]=%d out of range", t, e);
    bn.push_back(e);
    if (t < edgedist[3]) b2.push_back(e);
  }
  for (int e = 0; e < Ne; ++e)
    if (mark[e] < 0 || mark[e] > 6) return fail(ctx, SGPU_BAD_GRID, "mark[%d]=%d out of range", e, mark[e]);
  for (int b = 0; b < nb3; ++b) {
    const int i = ctx->dev2cell[ctx->ncomp + b];
    bnf[b] = ctx->nfaces[i];
    for (int f = 0; f < bnf[b]; ++f) {
      const int e = face[(size_t)i * F + f], v = normal[(size_t)i * F + f];
      if (e < 0 || e >= Ne) return fail(ctx, SGPU_BAD_GRID, "face[%d]=%d out of range", i * F + f, e);
      if (v != 1 && v != -1) return fail(ctx, SGPU_BAD_GRID, "normal[%d]=%d is not +1 or -1", i * F + f, v);
      bfe[(size_t)b * F + f] = e;
      bnr[(size_t)b * F + f] = v;
    }
  }
  DeviceGuard dg(ctx->device);
  int rc;
  if (!ctx->up_grid) {
    if ((rc = dalloc(ctx, &ctx->d_b2edge, (size_t)Ne + 1)) || (rc = dalloc(ctx, &ctx->d_bedge, (size_t)Ne + 1)) ||
        (rc = dalloc(ctx, &ctx->d_bnfaces, bnf.size())) || (rc = dalloc(ctx, &ctx->d_bfedge, bfe.size())) ||
        (rc = dalloc(ctx, &ctx->d_bnormal, bnr.size())) || (rc = dalloc(ctx, &ctx->d_mark, (size_t)Ne + 1)) ||
        (rc = dalloc(ctx, &ctx->d_n1, (size_t)Ne + 1)) || (rc = dalloc(ctx, &ctx->d_n2, (size_t)Ne + 1)))
      return rc;
  }
  if (!b2.empty()) CK(cudaMemcpyAsync(ctx->d_b2edge, b2.data(), sizeof(int) * b2.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (!bn.empty()) CK(cudaMemcpyAsync(ctx->d_bedge, bn.data(), sizeof(int) * bn.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_bnfaces, bnf.data(), sizeof(int) * bnf.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_bfedge, bfe.data(), sizeof(int) * bfe.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_bnormal, bnr.data(), sizeof(int) * bnr.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_mark, mark, sizeof(int) * Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_n1, n1, sizeof(double) * Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_n2, n2, sizeof(double) * Ne, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->nb2 = (int)b2.size();
  ctx->nbnd = (int)bn.size();
  ctx->up_grid = true;
  return SGPU_OK;
}

static int kmax_for(int Nkmax) {
  const int need = Nkmax + 1;
  return need <= 16 ? 16 : need <= 32 ? 32 : need <= 64 ? 64 : 128;
}

static UPredArgs upred_args(sgpu_context* ctx, const sgpu_props* p, const sgpu_upred_fields* f) {
  UPredArgs a{};
  a.Nc = ctx->Nc;
  a.Ne = ctx->Ne;
  a.ncomp = ctx->ncomp;
  a.ncell3 = ctx->nbdy;
  a.F = ctx->F;
  a.ncedge = ctx->ncedge;
  a.nb2 = ctx->nb2;
  a.nbnd = ctx->nbnd;
  a.kmax = kmax_for(ctx->Nkmax);
  a.dt = p->dt;
  a.theta = p->theta;
  a.grav = p->grav;
  if (f) {
    a.nu = f->nu;
    a.lax = f->laxWendroff_Vertical;
    a.thetaM = f->thetaM;
    a.nonlinear = f->nonlinear;
  }
  a.cedge = ctx->d_cedge;
  a.b2edge = ctx->d_b2edge;
  a.bedge = ctx->d_bedge;
  a.grad = ctx->d_grad;
  a.nke = ctx->d_nke;
  a.eoff = ctx->d_eoff;
  a.dcoff = ctx->d_dcoff;
  a.woff = ctx->d_woff;
  a.ctop = ctx->d_ctop;
  a.etop = ctx->d_etop;
  a.nfaces = ctx->d_nfaces;
  a.fedge = ctx->d_fedge;
  a.normal = ctx->d_normal;
  a.bnfaces = ctx->d_bnfaces;
  a.bfedge = ctx->d_bfedge;
  a.bnormal = ctx->d_bnormal;
  a.mark = ctx->d_mark;
  a.n1 = ctx->d_n1;
  a.n2 = ctx->d_n2;
  a.dzz = ctx->d_dzz;
  a.dzf = ctx->d_dzf;
  a.dg = ctx->d_dg;
  a.df = ctx->d_df;
  a.Ac = ctx->d_Ac;
  a.dv = ctx->d_dv;
  a.tau_T = ctx->d_tauT;
  a.CdT = ctx->d_CdT;
  a.CdB = ctx->d_CdB;
  a.nu_tv = ctx->d_nutv;
  a.nu_lax = ctx->d_nulax;
  a.w = ctx->d_w;
  a.u = ctx->d_u;
  a.h = ctx->d_hv;
  a.utmp = ctx->d_utmp;
  a.E = ctx->d_E;
  a.D = ctx->d_Dh;
  a.htmp = ctx->d_bin;
  a.u_out = ctx->d_u;
  a.active = ctx->d_active;
  a.nnan = ctx->d_nnan;
  return a;
}

static int upred_common_checks(sgpu_context* ctx) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  if (ctx->Nkmax + 1 > 128) return fail(ctx, SGPU_BAD_GRID, "UPredictor on the device needs Nkmax <= 127");
  DeviceGuard dg(ctx->device);
  int rc;
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx)) || (rc = alloc_vgrid(ctx)) || (rc = alloc_h(ctx)) ||
      (rc = alloc_upred(ctx)))
    return rc;
  return SGPU_OK;
}

static int check_etop(sgpu_context* ctx, const int* etop) {
  for (int e = 0; e < ctx->Ne; ++e)
    if (etop[e] < 0 || (ctx->Nke[e] > 0 && etop[e] >= ctx->Nke[e]) || (ctx->Nke[e] == 0 && etop[e] != 0))
      return fail(ctx, SGPU_BAD_ARG, "etop[%d]=%d out of [0,Nke)", e, etop[e]);
  return SGPU_OK;
}

// the inputs of the vertical predictor, staged and uploaded (ctop, etop, dzz,
// dzf, u, w, h, utmp and the drag / viscosity fields)
static int upload_upred_inputs(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                               const double* const* dzf, const double* h, const sgpu_upred_fields* f,
                               const double* const* utmp) {
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, nw3 = ctx->nw3, Nc = ctx->Nc, Ne = ctx->Ne, ni = (Nc + Ne + 1) / 2 + 1;
  int rc;
  if ((rc = ensure_pinned(ctx, ni + 3 * n3 + 3 * ne3 + nw3 + Nc + 3 * Ne + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  int* s_etop = s_ctop + Nc;
  double* s_dzz = ctx->pin + ni;
  double* s_nut = s_dzz + n3;
  double* s_nul = s_nut + n3;
  double* s_dzf = s_nul + n3;
  double* s_u = s_dzf + ne3;
  double* s_ut = s_u + ne3;
  double* s_w = s_ut + ne3;
  double* s_h = s_w + nw3;
  double* s_tc = s_h + Nc;
  for (size_t j = 0; j < Nc; ++j) {
    s_ctop[j] = ctop[ctx->dev2cell[j]];
    s_h[j] = h[ctx->dev2cell[j]];
  }
  std::memcpy(s_etop, etop, sizeof(int) * Ne);
  gather_cells(ctx, dzz, s_dzz);
  gather_cells(ctx, f->nu_tv, s_nut);
  gather_cells(ctx, f->nu_lax, s_nul);
  gather_edges(ctx, dzf, s_dzf);
  gather_edges(ctx, f->u, s_u);
  gather_edges(ctx, utmp, s_ut);
  const bool adv = f->nonlinear && f->thetaM >= 0;
  if (adv) gather_wrows(ctx, f->w, s_w);
  std::memcpy(s_tc, f->tau_T, sizeof(double) * Ne);
  std::memcpy(s_tc + Ne, f->CdT, sizeof(double) * Ne);
  std::memcpy(s_tc + 2 * Ne, f->CdB, sizeof(double) * Ne);
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * Nc, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_nutv, s_nut, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_nulax, s_nul, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_dzf, s_dzf, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_utmp, s_ut, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  if (adv) CK(cudaMemcpyAsync(ctx->d_w, s_w, sizeof(double) * nw3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_hv, s_h, sizeof(double) * Nc, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_tauT, s_tc, sizeof(double) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_CdT, s_tc + Ne, sizeof(double) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_CdB, s_tc + 2 * Ne, sizeof(double) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(ctx->d_nnan, 0, sizeof(int), st));
  return SGPU_OK;
}

static bool upred_fields_ok(const sgpu_upred_fields* f) {
  return f && f->u && f->nu_tv && f->nu_lax && f->tau_T && f->CdT && f->CdB &&
         (f->w || !(f->nonlinear && f->thetaM >= 0));
}

// E rows of the computational edges, from device staging to the caller's rows
static void scatter_cedge_rows(sgpu_context* ctx, const double* src, double* const* rows) {
  host_parallel((long long)ctx->cedge_h.size(), [&](long long b, long long e) {
    for (long long t = b; t < e; ++t) {
      const int k = ctx->cedge_h[t];
      std::memcpy(rows[k], src + ctx->eoff[k], sizeof(double) * ctx->Nke[k]);
    }
  });
}

int sgpu_upredictor_vertical(sgpu_context* ctx, const int* ctop, const int* etop, const double* const* dzz,
                             const double* const* dzf, const double* h, const sgpu_upred_fields* f,
                             const sgpu_props* prop, double* const* utmp, double* const* E, double* D) {
  int rc;
  if ((rc = upred_common_checks(ctx))) return rc;
  if (!ctop || !etop || !dzz || !dzf || !h || !upred_fields_ok(f) || !prop || !utmp || !E || !D)
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if ((rc = check_ctop(ctx, ctop)) || (rc = check_etop(ctx, etop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = upload_upred_inputs(ctx, ctop, etop, dzz, dzf, h, f, (const double* const*)utmp))) return rc;
  UPredArgs a = upred_args(ctx, prop, f);
  CK(launch_upred_vertical(a, ctx->stream));
  const size_t ne3 = ctx->ne3;
  double* s_ut = ctx->pin;
  double* s_E = s_ut + ne3;
  int nnan = 0;
  CK(cudaMemcpyAsync(s_ut, ctx->d_utmp, sizeof(double) * ne3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(s_E, ctx->d_E, sizeof(double) * ne3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(D, ctx->d_Dh, sizeof(double) * ctx->Ne, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(&nnan, ctx->d_nnan, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  scatter_edges(ctx, s_ut, utmp);
  scatter_cedge_rows(ctx, s_E, E);
  ctx->q_uploaded = false;
  ctx->h_uploaded = false;
  if (nnan) return fail(ctx, SGPU_BREAKDOWN, "U*** has %d NaN values (the reference stops here)", nnan);
  return SGPU_OK;
}

int sgpu_upredictor_rhs(sgpu_context* ctx, const int* etop, const double* const* dzf, const double* const* u,
                        const double* const* utmp, const double* h, const sgpu_props* prop, double* htmp) {
  int rc;
  if ((rc = upred_common_checks(ctx))) return rc;
  if (!etop || !dzf || !u || !utmp || !h || !prop || !htmp) return fail(ctx, SGPU_BAD_ARG, "null argument");
  if ((rc = check_etop(ctx, etop))) return rc;
  DeviceGuard dg(ctx->device);
  const size_t ne3 = ctx->ne3, Nc = ctx->Nc, Ne = ctx->Ne, ni = Ne / 2 + 1;
  if ((rc = ensure_pinned(ctx, ni + 3 * ne3 + 2 * Nc + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_etop = (int*)ctx->pin;
  double* s_dzf = ctx->pin + ni;
  double* s_u = s_dzf + ne3;
  double* s_ut = s_u + ne3;
  double* s_h = s_ut + ne3;
  std::memcpy(s_etop, etop, sizeof(int) * Ne);
  gather_edges(ctx, dzf, s_dzf);
  gather_edges(ctx, u, s_u);
  gather_edges(ctx, utmp, s_ut);
  for (size_t j = 0; j < Nc; ++j) s_h[j] = h[ctx->dev2cell[j]];
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_dzf, s_dzf, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_utmp, s_ut, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_hv, s_h, sizeof(double) * Nc, cudaMemcpyHostToDevice, st));
  UPredArgs a = upred_args(ctx, prop, nullptr);
  CK(launch_upred_rhs(a, st));
  double* s_b = s_h + Nc;
  CK(cudaMemcpyAsync(s_b, ctx->d_bin, sizeof(double) * ctx->ncomp, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int j = 0; j < ctx->ncomp; ++j) htmp[ctx->dev2cell[j]] = s_b[j];
  ctx->h_uploaded = false;
  return SGPU_OK;
}

// download of the state the finish step and the whole predictor leave
static int download_upred_state(sgpu_context* ctx, int* ctop, int* etop, double* const* dzz, double* h,
                                unsigned char* active, double* const* u) {
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, Nc = ctx->Nc, Ne = ctx->Ne, ni = (Nc + Ne + 1) / 2 + 1;
  int rc;
  if ((rc = ensure_pinned(ctx, ni + n3 + ne3 + 2 * Nc + 8))) return rc;
  int* o_ctop = (int*)ctx->pin;
  int* o_etop = o_ctop + Nc;
  double* s_dzz = ctx->pin + ni;
  double* s_u = s_dzz + n3;
  double* s_h = s_u + ne3;
  unsigned char* s_act = (unsigned char*)(s_h + Nc);
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(o_ctop, ctx->d_ctop, sizeof(int) * Nc, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(o_etop, ctx->d_etop, sizeof(int) * Ne, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_dzz, ctx->d_dzz, sizeof(double) * n3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_u, ctx->d_u, sizeof(double) * ne3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_h, ctx->d_hv, sizeof(double) * Nc, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_act, ctx->d_active, Nc, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (size_t j = 0; j < Nc; ++j) {
    const int i = ctx->dev2cell[j];
    ctop[i] = o_ctop[j];
    h[i] = s_h[j];
    active[i] = s_act[j];
  }
  std::memcpy(etop, o_etop, sizeof(int) * Ne);
  scatter_cells_all(ctx, s_dzz, dzz);
  scatter_edges(ctx, s_u, u);
  return SGPU_OK;
}

// dry-cell clip, u on computational edges, UpdateDZ, type-2 / type-3 boundaries
static cudaError_t launch_upred_finish(sgpu_context* ctx, const sgpu_vgrid* v, const UPredArgs& a) {
  cudaError_t e;
  if ((e = launch_upred_velocity(a, ctx->stream))) return e;
  VGridArgs va = vgrid_args(ctx, v, 0);
  if ((e = launch_update_dz(va, ctx->stream))) return e;
  return launch_upred_boundary(a, ctx->stream);
}

int sgpu_upredictor_finish(sgpu_context* ctx, const sgpu_vgrid* v, const sgpu_props* prop, int* ctop, int* etop,
                           double* const* dzz, const double* const* utmp, const double* const* E, double* h,
                           unsigned char* active, double* const* u) {
  int rc;
  if ((rc = upred_common_checks(ctx))) return rc;
  if (!v || !v->dz || !v->dv || !prop || !ctop || !etop || !dzz || !utmp || !E || !h || !active || !u)
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->up_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_upredictor_grid has not been called");
  if ((rc = check_ctop(ctx, ctop)) || (rc = check_etop(ctx, etop))) return rc;
  DeviceGuard dg(ctx->device);
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, Nc = ctx->Nc, Ne = ctx->Ne, ni = (Nc + Ne + 1) / 2 + 1;
  if ((rc = ensure_pinned(ctx, ni + n3 + 3 * ne3 + 3 * Nc + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  int* s_etop = s_ctop + Nc;
  double* s_dzz = ctx->pin + ni;
  double* s_ut = s_dzz + n3;
  double* s_E = s_ut + ne3;
  double* s_u = s_E + ne3;
  double* s_dv = s_u + ne3;
  double* s_dzbot = s_dv + Nc;
  double* s_h = s_dzbot + Nc;
  for (size_t j = 0; j < Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  std::memcpy(s_etop, etop, sizeof(int) * Ne);
  gather_cells(ctx, (const double* const*)dzz, s_dzz);
  gather_edges(ctx, utmp, s_ut);
  gather_edges(ctx, E, s_E);
  gather_edges(ctx, (const double* const*)u, s_u);
  if ((rc = upload_vgrid_common(ctx, v, h, s_dv, s_dzbot, s_h))) return rc;
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * Nc, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_etop, s_etop, sizeof(int) * Ne, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_utmp, s_ut, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_E, s_E, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_u, s_u, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  UPredArgs a = upred_args(ctx, prop, nullptr);
  CK(launch_upred_finish(ctx, v, a));
  CK(cudaStreamSynchronize(st));
  if ((rc = download_upred_state(ctx, ctop, etop, dzz, h, active, u))) return rc;
  ctx->q_uploaded = false;
  return SGPU_OK;
}

int sgpu_upredictor(sgpu_context* ctx, const sgpu_vgrid* v, const sgpu_upred_fields* f, const sgpu_props* prop,
                    int* ctop, int* etop, double* const* dzz, const double* const* dzf, double* const* u, double* h,
                    double* const* utmp, double* const* E, double* D, unsigned char* active, sgpu_stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  int rc;
  if ((rc = upred_common_checks(ctx))) return rc;
  if (!v || !v->dz || !v->dv || !upred_fields_ok(f) || !prop || !ctop || !etop || !dzz || !dzf || !u || !h ||
      !utmp || !E || !D || !active)
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->up_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_upredictor_grid has not been called");
  if ((rc = check_ctop(ctx, ctop)) || (rc = check_etop(ctx, etop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = upload_upred_inputs(ctx, ctop, etop, (const double* const*)dzz, dzf, h, f, (const double* const*)utmp)))
    return rc;
  {
    double* s_dv = ctx->pin + ((ctx->Nc + ctx->Ne + 1) / 2 + 1) + 3 * ctx->n3;  // staging behind the dzz block
    CK(cudaStreamSynchronize(ctx->stream));
    for (int j = 0; j < ctx->Nc; ++j) {
      const int i = ctx->dev2cell[j];
      s_dv[j] = v->dv[i];
      s_dv[ctx->Nc + j] = v->dzbot ? v->dzbot[i] : 0.0;
    }
    CK(cudaMemcpyAsync(ctx->d_dz, v->dz, sizeof(double) * ctx->Nkmax, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_dv, s_dv, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_dzbot, s_dv + ctx->Nc, sizeof(double) * ctx->Nc, cudaMemcpyHostToDevice, ctx->stream));
  }
  cudaStream_t st = ctx->stream;
  UPredArgs a = upred_args(ctx, prop, f);
  // U***, E, D
  CK(launch_upred_vertical(a, st));
  int nnan = 0;
  CK(cudaMemcpyAsync(&nnan, ctx->d_nnan, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (nnan) return fail(ctx, SGPU_BREAKDOWN, "U*** has %d NaN values (the reference stops here)", nnan);
  // BoundaryVelocities / OpenBoundaryFluxes without boundary data
  if (ctx->nbdy > 0) CK(cudaMemsetAsync(ctx->d_hv + ctx->ncomp, 0, sizeof(double) * ctx->nbdy, st));
  VGridArgs va = vgrid_args(ctx, v, 0);
  CK(launch_update_dz(va, st));
  CK(launch_upred_open_fluxes(a, st));
  // the free-surface right-hand side and CGSolve, all in HBM
  CK(launch_upred_rhs(a, st));
  CK(cudaMemcpyAsync(ctx->d_hin, ctx->d_hv, sizeof(double) * ctx->Nc, cudaMemcpyDeviceToDevice, st));
  ctx->h_uploaded = true;
  ctx->h_solved = false;
  int s_rc = sgpu_h_solve(ctx, prop, stats);
  if (s_rc != SGPU_OK && s_rc != SGPU_MAXITER && s_rc != SGPU_BREAKDOWN) return s_rc;
  if (ctx->ncomp > 0)
    CK(cudaMemcpyAsync(ctx->d_hv, ctx->d_hx, sizeof(double) * ctx->ncomp, cudaMemcpyDeviceToDevice, st));
  CK(launch_upred_finish(ctx, v, a));
  // results
  const size_t ne3 = ctx->ne3;
  if ((rc = download_upred_state(ctx, ctop, etop, dzz, h, active, u))) return rc;
  double* s_ut = ctx->pin;
  double* s_E = s_ut + ne3;
  CK(cudaMemcpyAsync(s_ut, ctx->d_utmp, sizeof(double) * ne3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_E, ctx->d_E, sizeof(double) * ne3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(D, ctx->d_Dh, sizeof(double) * ctx->Ne, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  scatter_edges(ctx, s_ut, utmp);
  scatter_cedge_rows(ctx, s_E, E);
  ctx->q_uploaded = false;
  ctx->h_uploaded = false;
  if (stats) stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return s_rc;
}

// ---------------------------------------------------------------------------
// WPredictor
// ---------------------------------------------------------------------------
static int alloc_wpred(sgpu_context* ctx) {
  if (ctx->wp_ready) return SGPU_OK;
  int rc;
  const size_t n3 = ctx->n3 + 1, ne3 = ctx->ne3 + 1;
  if ((rc = dalloc(ctx, &ctx->d_cnw, n3)) || (rc = dalloc(ctx, &ctx->d_cnw2, n3)) || (rc = dalloc(ctx, &ctx->d_wt, n3)) ||
      (rc = dalloc(ctx, &ctx->d_wcc, n3)) || (rc = dalloc(ctx, &ctx->d_wface, ne3)))
    return rc;
  ctx->wp_ready = true;
  return SGPU_OK;
}

static WPredArgs wpred_args(sgpu_context* ctx, const sgpu_wpred_fields* f, const sgpu_props* prop) {
  WPredArgs a{};
  a.Nc = ctx->Nc;
  a.ncomp = ctx->ncomp;
  a.F = ctx->F;
  a.ncedge = ctx->ncedge;
  a.kmax = kmax_for(ctx->Nkmax);
  a.n3 = (int)ctx->n3;
  a.nonlinear = f->nonlinear;
  a.first = f->n == 1;
  if (f->n == 1) {  // main/phys.c:2044-2064
    a.fab1 = 1;
    a.fab2 = a.fab3 = 0;
  } else if (f->n == 2 || f->AB == 2) {
    a.fab1 = 3.0 / 2.0;
    a.fab2 = -1.0 / 2.0;
    a.fab3 = 0;
  } else {
    a.fab1 = 23.0 / 12.0;
    a.fab2 = -4.0 / 3.0;
    a.fab3 = 5.0 / 12.0;
  }
  a.dt = prop->dt;
  a.theta = prop->theta;
  a.nu = f->nu;
  a.nu_H = f->nu_H;
  a.CdW = f->CdW;
  a.lax = f->laxWendroff_Vertical;
  a.cedge = ctx->d_cedge;
  a.grad = ctx->d_grad;
  a.nke = ctx->d_nke;
  a.eoff = ctx->d_eoff;
  a.dcoff = ctx->d_dcoff;
  a.woff = ctx->d_woff;
  a.nk = ctx->d_nk;
  a.ctop = ctx->d_ctop;
  a.nfaces = ctx->d_nfaces;
  a.fedge = ctx->d_fedge;
  a.normal = ctx->d_normal;
  a.ecsr = ctx->d_ecsr;
  a.eside = ctx->d_eside;
  a.dzz = ctx->d_dzz;
  a.df = ctx->d_df;
  a.dg = ctx->d_dg;
  a.Ac = ctx->d_Ac;
  a.q = ctx->d_qtot;
  a.nu_tv = ctx->d_nutv;
  a.nu_lax = ctx->d_nulax;
  a.utmp2 = ctx->d_ut2;
  a.w = ctx->d_w;
  a.Cn_W = ctx->d_cnw;
  a.Cn_W2 = ctx->d_cnw2;
  a.wtmp = ctx->d_wt;
  a.wc = ctx->d_wcc;
  a.ut = ctx->d_wface;
  return a;
}

int sgpu_wpredictor(sgpu_context* ctx, const int* ctop, const double* const* dzz, const sgpu_wpred_fields* f,
                    const sgpu_props* prop, double* const* w, double* const* Cn_W, double* const* Cn_W2) {
  if (!ctx || !ctx->stream) return ctx ? fail(ctx, SGPU_NO_DEVICE, "context has no device state") : SGPU_BAD_ARG;
  if (!ctop || !dzz || !f || !f->q || !f->nu_tv || !f->nu_lax || !prop || !w || !Cn_W || !Cn_W2 ||
      (f->nonlinear && !f->utmp2))
    return fail(ctx, SGPU_BAD_ARG, "null argument");
  if (!ctx->step_grid) return fail(ctx, SGPU_BAD_ARG, "sgpu_step_grid has not been called");
  if (f->nonlinear != 0 && f->nonlinear != 1)
    return fail(ctx, SGPU_BAD_ARG, "WPredictor on the device supports nonlinear 0 and 1, not %d", f->nonlinear);
  if (f->conserveMomentum) return fail(ctx, SGPU_BAD_ARG, "WPredictor on the device needs conserveMomentum 0");
  if (ctx->Nkmax + 1 > 128) return fail(ctx, SGPU_BAD_GRID, "WPredictor on the device needs Nkmax <= 127");
  if (ctx->F > 8) return fail(ctx, SGPU_BAD_GRID, "WPredictor on the device needs maxfaces <= 8");
  int rc;
  if ((rc = check_ctop(ctx, ctop))) return rc;
  DeviceGuard dg(ctx->device);
  if ((rc = alloc_q(ctx)) || (rc = alloc_step(ctx)) || (rc = alloc_upred(ctx)) || (rc = alloc_wpred(ctx))) return rc;
  const size_t n3 = ctx->n3, ne3 = ctx->ne3, nw3 = ctx->nw3, Nc = ctx->Nc, ni = Nc / 2 + 1;
  if ((rc = ensure_pinned(ctx, ni + 6 * n3 + ne3 + nw3 + 8))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  int* s_ctop = (int*)ctx->pin;
  double* s_dzz = ctx->pin + ni;
  double* s_q = s_dzz + n3;
  double* s_nt = s_q + n3;
  double* s_nl = s_nt + n3;
  double* s_c1 = s_nl + n3;
  double* s_c2 = s_c1 + n3;
  double* s_u2 = s_c2 + n3;
  double* s_w = s_u2 + ne3;
  for (size_t j = 0; j < Nc; ++j) s_ctop[j] = ctop[ctx->dev2cell[j]];
  gather_cells(ctx, dzz, s_dzz);
  gather_cells(ctx, f->q, s_q);
  gather_cells(ctx, f->nu_tv, s_nt);
  gather_cells(ctx, f->nu_lax, s_nl);
  gather_cells(ctx, (const double* const*)Cn_W, s_c1);
  gather_cells(ctx, (const double* const*)Cn_W2, s_c2);
  if (f->nonlinear) gather_edges(ctx, f->utmp2, s_u2);
  gather_wrows(ctx, (const double* const*)w, s_w);
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(ctx->d_ctop, s_ctop, sizeof(int) * Nc, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_dzz, s_dzz, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_qtot, s_q, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_nutv, s_nt, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_nulax, s_nl, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_cnw, s_c1, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_cnw2, s_c2, sizeof(double) * n3, cudaMemcpyHostToDevice, st));
  if (f->nonlinear) CK(cudaMemcpyAsync(ctx->d_ut2, s_u2, sizeof(double) * ne3, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->d_w, s_w, sizeof(double) * nw3, cudaMemcpyHostToDevice, st));
  WPredArgs a = wpred_args(ctx, f, prop);
  if (f->nonlinear) CK(cudaMemsetAsync(ctx->d_wface, 0, sizeof(double) * ne3, st));
  CK(launch_wpredictor(a, st));
  CK(cudaMemcpyAsync(s_w, ctx->d_w, sizeof(double) * nw3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_c1, ctx->d_cnw, sizeof(double) * n3, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(s_c2, ctx->d_cnw2, sizeof(double) * n3, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  scatter_wrows(ctx, s_w, w, ctx->ncomp);
  scatter_cells_all(ctx, s_c1, Cn_W);
  scatter_cells_all(ctx, s_c2, Cn_W2);
  ctx->q_uploaded = false;
  return SGPU_OK;
}

}  // extern "C"
