// ztm_capi.cu - the C ABI (include/ztm_grav.h): context lifetime, argument
// checks, host<->device staging and dispatch to the kernels.
//
// The reference boundary this replaces is a process boundary: TFM.cpp:90-94
// writes float32 files to /dev/shm, runs ./GFM, and GFM_GPU.cu:24-34 creates
// a CUDA context, copies, launches GF and writes G.dat back on every call.
// Here the context (device, stream, workspace) persists across calls and
// the data crosses as plain pointers.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "ztm_internal.cuh"

namespace {

struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = (cudaSetDevice(dev) == cudaSuccess);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
      cudaSetDevice(prev);
  }
};

inline bool is_dev(int flags) { return (flags & ZTM_FLAG_DEVICE_PTRS) != 0; }

double pick_G(const ztm_opts* o) {
  return (o && o->G > 0) ? o->G : 6.67e-11;
}

int check_opts(ztm_ctx* c, const ztm_opts* o) {
  if (!o) return ZTM_OK;
  if (o->precision < ZTM_PREC_FP64 || o->precision > ZTM_PREC_MIXED)
    return ztm_fail(c, ZTM_ERR_ARG, "opts.precision must be 0, 1 or 2");
  if (o->flags & ~(ZTM_FLAG_DEVICE_PTRS | ZTM_FLAG_AUTOTUNE))
    return ztm_fail(c, ZTM_ERR_ARG, "unknown bit in opts.flags");
  if (!(o->G >= 0) || !(o->near_q >= 0) || o->tile < 0 || o->chunk < 0)
    return ztm_fail(c, ZTM_ERR_ARG, "negative or NaN option value");
  if (o->tile && (o->tile % 32 || o->tile > 512))
    return ztm_fail(c, ZTM_ERR_ARG, "opts.tile must be a multiple of 32, <= 512");
  return ZTM_OK;
}

int check_mesh(ztm_ctx* c, const ztm_mesh* m) {
  if (!m) return ztm_fail(c, ZTM_ERR_ARG, "mesh is NULL");
  if (m->nx < 1 || m->ny < 1 || m->nz < 1)
    return ztm_fail(c, ZTM_ERR_ARG, "mesh dimensions must be >= 1");
  if ((long long)m->nx * m->ny * m->nz > (1LL << 31) - 1)
    return ztm_fail(c, ZTM_ERR_RANGE, "mesh has more than 2^31-1 prisms");
  if (!(m->dx > 0) || !(m->dy > 0) || !(m->dz > 0))
    return ztm_fail(c, ZTM_ERR_ARG, "mesh cell sizes must be > 0");
  if (!isfinite(m->x0) || !isfinite(m->y0) || !isfinite(m->z_top))
    return ztm_fail(c, ZTM_ERR_ARG, "mesh origin must be finite");
  return ZTM_OK;
}

int check_imesh(ztm_ctx* c, const ztm_imesh* m) {
  if (!m) return ztm_fail(c, ZTM_ERR_ARG, "interface mesh is NULL");
  if (m->nx < 1 || m->ny < 1)
    return ztm_fail(c, ZTM_ERR_ARG, "interface mesh dimensions must be >= 1");
  if ((long long)m->nx * m->ny > (1LL << 31) - 1)
    return ztm_fail(c, ZTM_ERR_RANGE, "interface mesh too large");
  if (!(m->dx > 0) || !(m->dy > 0))
    return ztm_fail(c, ZTM_ERR_ARG, "interface cell sizes must be > 0");
  if (!isfinite(m->x0) || !isfinite(m->y0) || !isfinite(m->z_base))
    return ztm_fail(c, ZTM_ERR_ARG, "interface origin must be finite");
  return ZTM_OK;
}

MeshDesc to_desc(const ztm_mesh* m) {
  MeshDesc d;
  d.nx = m->nx; d.ny = m->ny; d.nz = m->nz;
  d.x0 = m->x0; d.y0 = m->y0; d.zt = m->z_top;
  d.dx = m->dx; d.dy = m->dy; d.dz = m->dz;
  return d;
}

IMeshDesc to_idesc(const ztm_imesh* m) {
  IMeshDesc d;
  d.nx = m->nx; d.ny = m->ny; d.x0 = m->x0; d.y0 = m->y0;
  d.dx = m->dx; d.dy = m->dy; d.zb = m->z_base;
  return d;
}

// Finish a call: copy out (host mode), synchronise, check device errors.
int finish(ztm_ctx* c, bool dev, void* host_out, const void* dev_out,
           size_t bytes, const char* what) {
  int rc = ztm_after_launch(c, what);
  if (rc) return rc;
  if (!dev) {
    if (host_out && bytes) {
      rc = ztm_cuda_check(c, cudaMemcpyAsync(host_out, dev_out, bytes,
                                             cudaMemcpyDeviceToHost, c->stream),
                          "copy result to host");
      if (rc) return rc;
    }
    rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), what);
    if (rc) return rc;
    return ztm_check_device_error(c);
  }
  return ZTM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// shared host helpers (declared in ztm_internal.cuh)
int ztm_finish(ztm_ctx* c, bool dev, void* host_out, const void* dev_out, size_t bytes,
               const char* what) {
  return finish(c, dev, host_out, dev_out, bytes, what);
}

int ztm_pm_setup(ztm_ctx* c, const ztm_grid* g, PmParams* p) {
  if (g->di < 1 || g->dj < 1 || g->dk < 1 || g->fh < 1 || g->fv < 1 || g->bfr < 0)
    return ztm_fail(c, ZTM_ERR_ARG, "grid dims must be >= 1 and bfr >= 0");
  if (!(g->threshold >= 0) || !isfinite(g->scale))
    return ztm_fail(c, ZTM_ERR_ARG, "bad threshold or scale");
  p->di = g->di; p->dj = g->dj; p->fh = g->fh; p->fv = g->fv; p->bfr = g->bfr;
  p->ii = (g->di - 1) * g->fh + 1;
  p->jj = (g->dj - 1) * g->fh + 1;
  p->kk = (g->dk - 1) * g->fv + 1;
  p->N = (long long)p->ii * p->jj * p->kk;
  if (p->N > (1LL << 31) - 1)
    return ztm_fail(c, ZTM_ERR_RANGE, "fine grid exceeds 2^31-1 nodes");
  p->ni = std::max(0, g->di - 2 * g->bfr);
  p->nj = std::max(0, g->dj - 2 * g->bfr);
  p->ns = p->ni * p->nj;
  p->thr = g->threshold;
  p->nnodes = p->N;
  return ZTM_OK;
}

int ztm_fail(ztm_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int ztm_cuda_check(ztm_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ZTM_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  int code = (e == cudaErrorMemoryAllocation) ? ZTM_ERR_ALLOC : ZTM_ERR_CUDA;
  return ztm_fail(c, code, m);
}

int ztm_ws_reserve(ztm_ctx* c, size_t bytes) {
  if (bytes <= c->ws_size) return ZTM_OK;
  int rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "sync before workspace growth");
  if (rc) return rc;
  if (c->ws) cudaFree(c->ws);
  c->ws = nullptr;
  c->ws_size = 0;
  size_t want = bytes + bytes / 8;  // headroom against small growth
  if (cudaMalloc((void**)&c->ws, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc((void**)&c->ws, bytes) != cudaSuccess) {
      cudaGetLastError();
      c->ws = nullptr;
      return ztm_fail(c, ZTM_ERR_ALLOC,
                      "workspace allocation of " + std::to_string(bytes) + " bytes failed");
    }
    want = bytes;
  }
  c->ws_size = want;
  return ZTM_OK;
}

void ztm_fork(ztm_ctx* c) {
  cudaEventRecord(c->ev_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
}

void ztm_join(ztm_ctx* c) {
  cudaEventRecord(c->ev_join, c->aux);
  cudaStreamWaitEvent(c->stream, c->ev_join, 0);
}

int ztm_after_launch(ztm_ctx* c, const char* what) {
  return ztm_cuda_check(c, cudaGetLastError(), what);
}

int ztm_check_device_error(ztm_ctx* c) {
  int h = 0;
  int rc = ztm_cuda_check(c, cudaMemcpy(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost),
                          "read device error word");
  if (rc) return rc;
  if (h == 0) return ZTM_OK;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaStreamSynchronize(c->stream);
  if (h & ZTM_DEVERR_TIMEOUT)
    return ztm_fail(c, ZTM_ERR_TIMEOUT, "a bounded device-side wait gave up");
  return ztm_fail(c, ZTM_ERR_RANGE, "a device-side bounds check failed");
}

int ztm_stage_in(ztm_ctx* c, const void* src, size_t bytes, bool dev,
                 void* staged, const void** out) {
  if (dev || bytes == 0) {
    *out = src;
    return ZTM_OK;
  }
  *out = staged;
  return ztm_cuda_check(c, cudaMemcpyAsync(staged, src, bytes, cudaMemcpyHostToDevice,
                                           c->stream),
                        "copy input to device");
}

// ---------------------------------------------------------------------------
// C ABI
extern "C" {

int ztm_version(void) { return ZTM_VERSION; }

int ztm_ctx_create(int device, ztm_ctx** out) {
  if (!out) return ZTM_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return ZTM_ERR_NODEV;
  }
  if (device < 0 || device >= n) return ZTM_ERR_NODEV;
  ztm_ctx* c = new (std::nothrow) ztm_ctx();
  if (!c) return ZTM_ERR_ALLOC;
  c->device = device;
  DeviceGuard g(device);
  if (!g.ok) {
    delete c;
    return ZTM_ERR_NODEV;
  }
  int lo_prio = 0, hi_prio = 0;
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      // the side stream carries the short double near-field kernels that run
      // beside the float far-field kernels: give it the highest priority so
      // its blocks are placed first whenever a slot frees up
      cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, hi_prio) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaMalloc((void**)&c->d_err, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->d_err) cudaFree(c->d_err);
    delete c;
    return ZTM_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return ZTM_OK;
}

void ztm_ctx_destroy(ztm_ctx* c) {
  if (!c) return;
  DeviceGuard g(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& e : c->graphs) {
    if (e.exec) cudaGraphExecDestroy(e.exec);
    if (e.graph) cudaGraphDestroy(e.graph);
  }
  for (auto& r : c->prof_recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : c->prof_pool) cudaEventDestroy(e);
  if (c->ws) cudaFree(c->ws);
  if (c->d_err) cudaFree(c->d_err);
  if (c->d_forms) cudaFree(c->d_forms);
  if (c->aux) {
    cudaStreamSynchronize(c->aux);
    cudaStreamDestroy(c->aux);
  }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

const char* ztm_last_error(const ztm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int ztm_ctx_set_stream(ztm_ctx* c, void* stream) {
  if (!c) return ZTM_ERR_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return ZTM_OK;
}

void* ztm_ctx_stream(ztm_ctx* c) { return c ? (void*)c->stream : nullptr; }

long long ztm_ctx_launches(const ztm_ctx* c) { return c ? c->launches : -1; }

int ztm_ctx_tuning(const ztm_ctx* c, int* rows, int max_rows) {
  if (!c || max_rows < 0 || (max_rows > 0 && !rows)) return ZTM_ERR_ARG;
  int n = 0;
  for (const auto& r : c->tune_log) {
    if (n >= max_rows) break;
    for (int j = 0; j < 4; j++) rows[4 * n + j] = j < (int)r.size() ? r[j] : 0;
    n++;
  }
  return n;
}

int ztm_ctx_test_timeout(ztm_ctx* c, unsigned int polls) {
  if (!c) return ZTM_ERR_ARG;
  c->stage_wait_limit = polls;
  return ZTM_OK;
}

int ztm_ctx_count_forms(ztm_ctx* c, int enable) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (enable && !c->d_forms) {
    DeviceGuard g(c->device);
    if (cudaMalloc((void**)&c->d_forms, 4 * sizeof(unsigned long long)) != cudaSuccess) {
      cudaGetLastError();
      c->d_forms = nullptr;
      return ztm_fail(c, ZTM_ERR_ALLOC, "form counters");
    }
    if (cudaMemsetAsync(c->d_forms, 0, 4 * sizeof(unsigned long long), c->stream) != cudaSuccess)
      return ztm_fail(c, ZTM_ERR_CUDA, "form counters");
  }
  c->count_forms = enable != 0;
  return ZTM_OK;
}

int ztm_ctx_form_counts(ztm_ctx* c, long long* counts) {
  if (!c || !counts) return ZTM_ERR_ARG;
  c->err.clear();
  for (int j = 0; j < 4; j++) counts[j] = 0;
  if (!c->d_forms) return ZTM_OK;
  DeviceGuard g(c->device);
  unsigned long long h[4] = {0, 0, 0, 0};
  int rc = ztm_cuda_check(c, cudaMemcpyAsync(h, c->d_forms, sizeof h, cudaMemcpyDeviceToHost,
                                             c->stream),
                          "read form counters");
  if (!rc) rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "read form counters");
  if (rc) return rc;
  cudaMemsetAsync(c->d_forms, 0, sizeof h, c->stream);
  for (int j = 0; j < 4; j++) counts[j] = (long long)h[j];
  return ZTM_OK;
}

int ztm_ctx_sync(ztm_ctx* c) {
  if (!c) return ZTM_ERR_ARG;
  DeviceGuard g(c->device);
  int rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "stream synchronise");
  if (rc) return rc;
  return ztm_check_device_error(c);
}

// ---- point mass -----------------------------------------------------------
int ztm_gfm_pointmass(ztm_ctx* c, const ztm_grid* g, const double* drho,
                      const int* nn, long long n_nn, const double* surf,
                      double* G, int precision, int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!g || !drho || !surf || !G) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32)
    return ztm_fail(c, ZTM_ERR_ARG, "point-mass precision must be FP64 or FP32");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  PmParams p;
  int rc = ztm_pm_setup(c, g, &p);
  if (rc) return rc;
  const long long N = p.N;
  if (nn && n_nn < 0) return ztm_fail(c, ZTM_ERR_ARG, "n_nn < 0");
  p.nnodes = nn ? n_nn : N;
  const bool dev = is_dev(flags);
  if (nn && !dev) {
    for (long long t = 0; t < n_nn; t++)
      if (nn[t] < 0 || nn[t] >= N)
        return ztm_fail(c, ZTM_ERR_RANGE, "nn[" + std::to_string(t) + "] outside the fine grid");
  }
  const long long M = (long long)g->di * g->dj;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = WsCarver::need(N * 8) + WsCarver::need((nn ? n_nn : 0) * 4) +
                2 * WsCarver::need(M * 8) + ztm_pointmass_ws(p, precision, c->num_sms) + 4096;
  rc = ztm_ws_reserve(c, need);
  if (rc) return rc;
  WsCarver wc(c->ws);
  double* s_drho = wc.take<double>(N);
  int* s_nn = wc.take<int>(nn ? n_nn : 0);
  double* s_surf = wc.take<double>(M);
  double* s_G = wc.take<double>(M);
  const void *pd, *pn = nullptr, *ps;
  if ((rc = ztm_stage_in(c, drho, N * 8, dev, s_drho, &pd))) return rc;
  if (nn && (rc = ztm_stage_in(c, nn, n_nn * 4, dev, s_nn, &pn))) return rc;
  if ((rc = ztm_stage_in(c, surf, M * 8, dev, s_surf, &ps))) return rc;
  double* outG = dev ? G : s_G;
  rc = ztm_launch_pointmass(c, p, (const double*)pd, (const int*)pn, (const double*)ps, outG,
                            g->scale, precision, wc);
  if (rc) return rc;
  return finish(c, dev, G, outG, M * 8, "point-mass forward");
}

// ---- prism mesh -----------------------------------------------------------
int ztm_gfm_prism(ztm_ctx* c, const ztm_mesh* mesh, const double* rho, int ns,
                  const double* sxyz, double* gz, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_mesh(c, mesh)) || (rc = check_opts(c, o))) return rc;
  if (ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "ns < 0");
  if (ns == 0) return ZTM_OK;
  if (!rho || !sxyz || !gz) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  MeshDesc m = to_desc(mesh);
  long long np = (long long)m.nx * m.ny * m.nz;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = WsCarver::need(np * 8) + WsCarver::need((size_t)ns * 24) +
                WsCarver::need((size_t)ns * 8) + ztm_prism_ws(m, ns, prec, c->num_sms, o) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_rho = wc.take<double>(np);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_gz = wc.take<double>(ns);
  const void *pr, *px;
  if ((rc = ztm_stage_in(c, rho, np * 8, dev, s_rho, &pr))) return rc;
  if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
  double* out = dev ? gz : s_gz;
  rc = ztm_launch_prism(c, m, (const double*)pr, ns, (const double*)px, out, pick_G(o), prec, o,
                        wc);
  if (rc) return rc;
  return finish(c, dev, gz, out, (size_t)ns * 8, "prism forward");
}

int ztm_gfm_prism_list(ztm_ctx* c, long long np, const double* geom,
                       const double* rho, int ns, const double* sxyz,
                       double* gz, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_opts(c, o))) return rc;
  if (np < 0 || ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "negative size");
  if (np > (1LL << 31) - 1) return ztm_fail(c, ZTM_ERR_RANGE, "more than 2^31-1 prisms");
  if (ns == 0) return ZTM_OK;
  if (!sxyz || !gz || (np > 0 && (!geom || !rho)))
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  double nq = (o && o->near_q > 0) ? o->near_q : 6.0;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = WsCarver::need(np * 48) + WsCarver::need(np * 8) +
                WsCarver::need((size_t)ns * 24) + WsCarver::need((size_t)ns * 8) +
                ztm_prism_list_ws(np, ns, prec, c->num_sms) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_geom = wc.take<double>(np * 6);
  double* s_rho = wc.take<double>(np);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_gz = wc.take<double>(ns);
  const void *pg = nullptr, *pr = nullptr, *px;
  if (np > 0) {
    if ((rc = ztm_stage_in(c, geom, np * 48, dev, s_geom, &pg))) return rc;
    if ((rc = ztm_stage_in(c, rho, np * 8, dev, s_rho, &pr))) return rc;
  }
  if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
  double* out = dev ? gz : s_gz;
  rc = ztm_launch_prism_list(c, np, (const double*)pg, (const double*)pr, ns, (const double*)px,
                             out, pick_G(o), prec, nq, wc);
  if (rc) return rc;
  return finish(c, dev, gz, out, (size_t)ns * 8, "prism-list forward");
}

int ztm_gfm_adjoint(ztm_ctx* c, const ztm_mesh* mesh, int ns, const double* sxyz,
                    const double* resid, double* g_rho, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_mesh(c, mesh)) || (rc = check_opts(c, o))) return rc;
  if (ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "ns < 0");
  if (!g_rho || (ns > 0 && (!sxyz || !resid))) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  MeshDesc m = to_desc(mesh);
  long long np = (long long)m.nx * m.ny * m.nz;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = WsCarver::need((size_t)ns * 24) + WsCarver::need((size_t)ns * 8) +
                WsCarver::need(np * 8) + ztm_adjoint_ws(m, ns, prec, c->num_sms, o ? o->near_q : 0.0) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_res = wc.take<double>(ns);
  double* s_g = wc.take<double>(np);
  const void *px = nullptr, *pr = nullptr;
  if (ns > 0) {
    if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
    if ((rc = ztm_stage_in(c, resid, (size_t)ns * 8, dev, s_res, &pr))) return rc;
  }
  double* out = dev ? g_rho : s_g;
  rc = ztm_launch_adjoint(c, m, ns, (const double*)px, (const double*)pr, out, pick_G(o), prec, o,
                          wc);
  if (rc) return rc;
  return finish(c, dev, g_rho, out, np * 8, "prism adjoint");
}

// ---- interface ------------------------------------------------------------
int ztm_gfm_interface(ztm_ctx* c, const ztm_imesh* mesh, const double* depth,
                      const double* rho_col, int ns, const double* sxyz,
                      double* gz, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_imesh(c, mesh)) || (rc = check_opts(c, o))) return rc;
  if (ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "ns < 0");
  if (ns == 0) return ZTM_OK;
  if (!depth || !rho_col || !sxyz || !gz) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  IMeshDesc m = to_idesc(mesh);
  long long nc = (long long)m.nx * m.ny;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = 2 * WsCarver::need(nc * 8) + WsCarver::need((size_t)ns * 24) +
                WsCarver::need((size_t)ns * 8) + ztm_iface_ws(m, ns, prec, c->num_sms) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_dep = wc.take<double>(nc);
  double* s_rho = wc.take<double>(nc);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_gz = wc.take<double>(ns);
  const void *pd, *pr, *px;
  if ((rc = ztm_stage_in(c, depth, nc * 8, dev, s_dep, &pd))) return rc;
  if ((rc = ztm_stage_in(c, rho_col, nc * 8, dev, s_rho, &pr))) return rc;
  if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
  double* out = dev ? gz : s_gz;
  rc = ztm_launch_iface_fwd(c, m, (const double*)pd, (const double*)pr, ns, (const double*)px, out,
                            pick_G(o), prec, o, wc);
  if (rc) return rc;
  return finish(c, dev, gz, out, (size_t)ns * 8, "interface forward");
}

int ztm_gfm_interface_jvp(ztm_ctx* c, const ztm_imesh* mesh, const double* depth,
                          const double* rho_col, const double* d_depth, int ns,
                          const double* sxyz, double* dgz, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_imesh(c, mesh)) || (rc = check_opts(c, o))) return rc;
  if (ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "ns < 0");
  if (ns == 0) return ZTM_OK;
  if (!depth || !rho_col || !d_depth || !sxyz || !dgz)
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  IMeshDesc m = to_idesc(mesh);
  long long nc = (long long)m.nx * m.ny;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = 3 * WsCarver::need(nc * 8) + WsCarver::need((size_t)ns * 24) +
                WsCarver::need((size_t)ns * 8) + ztm_iface_ws(m, ns, prec, c->num_sms) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_dep = wc.take<double>(nc);
  double* s_rho = wc.take<double>(nc);
  double* s_v = wc.take<double>(nc);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_out = wc.take<double>(ns);
  const void *pd, *pr, *pv, *px;
  if ((rc = ztm_stage_in(c, depth, nc * 8, dev, s_dep, &pd))) return rc;
  if ((rc = ztm_stage_in(c, rho_col, nc * 8, dev, s_rho, &pr))) return rc;
  if ((rc = ztm_stage_in(c, d_depth, nc * 8, dev, s_v, &pv))) return rc;
  if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
  double* out = dev ? dgz : s_out;
  rc = ztm_launch_iface_jvp(c, m, (const double*)pd, (const double*)pr, (const double*)pv, ns,
                            (const double*)px, out, pick_G(o), prec, o, wc);
  if (rc) return rc;
  return finish(c, dev, dgz, out, (size_t)ns * 8, "interface depth derivative");
}

int ztm_gfm_interface_adjoint(ztm_ctx* c, const ztm_imesh* mesh, const double* depth,
                              const double* rho_col, int ns, const double* sxyz,
                              const double* resid, double* g_rho, double* g_depth,
                              const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  int rc;
  if ((rc = check_imesh(c, mesh)) || (rc = check_opts(c, o))) return rc;
  if (ns < 0) return ztm_fail(c, ZTM_ERR_ARG, "ns < 0");
  if (!depth || !rho_col || (ns > 0 && (!sxyz || !resid)))
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (!g_rho && !g_depth) return ZTM_OK;
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && is_dev(o->flags);
  IMeshDesc m = to_idesc(mesh);
  long long nc = (long long)m.nx * m.ny;
  DeviceGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = 4 * WsCarver::need(nc * 8) + WsCarver::need((size_t)ns * 24) +
                WsCarver::need((size_t)ns * 8) + ztm_iface_ws(m, ns, prec, c->num_sms) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_dep = wc.take<double>(nc);
  double* s_rho = wc.take<double>(nc);
  double* s_gr = wc.take<double>(nc);
  double* s_gd = wc.take<double>(nc);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_res = wc.take<double>(ns);
  const void *pd, *pr, *px = nullptr, *pres = nullptr;
  if ((rc = ztm_stage_in(c, depth, nc * 8, dev, s_dep, &pd))) return rc;
  if ((rc = ztm_stage_in(c, rho_col, nc * 8, dev, s_rho, &pr))) return rc;
  if (ns > 0) {
    if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
    if ((rc = ztm_stage_in(c, resid, (size_t)ns * 8, dev, s_res, &pres))) return rc;
  }
  double* ogr = g_rho ? (dev ? g_rho : s_gr) : nullptr;
  double* ogd = g_depth ? (dev ? g_depth : s_gd) : nullptr;
  rc = ztm_launch_iface_adj(c, m, (const double*)pd, (const double*)pr, ns, (const double*)px,
                            (const double*)pres, ogr, ogd, pick_G(o), prec, o, wc);
  if (rc) return rc;
  if (!dev && g_rho) {
    rc = ztm_cuda_check(c, cudaMemcpyAsync(g_rho, ogr, nc * 8, cudaMemcpyDeviceToHost, c->stream),
                        "copy g_rho");
    if (rc) return rc;
  }
  return finish(c, dev, g_depth, ogd, g_depth ? nc * 8 : 0, "interface adjoint");
}

}  // extern "C"
