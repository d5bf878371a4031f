// ztm_internal.cuh - context, workspace and device helpers shared by the
// gravity kernels.  Everything here is internal to libztmgrav.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/ztm_grav.h"

#define ZTM_VERSION 100

// Bounded spin limits (iterations of mbarrier try_wait).  A wait that runs
// out sets the context's device error word and the kernel returns.
#define ZTM_WAIT_LIMIT (1u << 24)
#define ZTM_DEVERR_TIMEOUT 1
#define ZTM_DEVERR_BOUNDS 2

struct ZtmGraphEntry {
  std::vector<long long> key;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

struct ZtmProfRec {
  const char* name;
  cudaEvent_t a, b;
};

struct ztm_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;  // side stream for concurrent kernels
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::string err;
  long long launches = 0;
  // grow-only device workspace; carved per call
  char* ws = nullptr;
  size_t ws_size = 0;
  // device error word written by bounded waits / bounds checks
  int* d_err = nullptr;
  // batched-launch graph cache and the host copy of the last job table
  std::vector<ZtmGraphEntry> graphs;
  std::vector<char> batch_table;
  // launch shapes chosen by the autotuner, keyed by workload shape, and the
  // timings of the candidates it measured ({shape..., microseconds})
  std::map<std::vector<long long>, std::vector<int>> tuned;
  std::vector<std::vector<int>> tune_log;
  // timeout-path test hook (ztm_ctx_test_timeout): polls of the far
  // kernel's redirected stage wait, 0 = off
  unsigned stage_wait_limit = 0;
  // evaluation-form counters of the mixed forward (ztm_ctx_count_forms)
  bool count_forms = false;
  unsigned long long* d_forms = nullptr;  // 4 counters on the device
  // tracing: events around compute kernels while enabled
  bool prof = false;
  std::vector<ZtmProfRec> prof_recs;
  std::vector<cudaEvent_t> prof_pool;
};

// Brackets one kernel launch with events when tracing is enabled.
struct ZtmProf {
  ztm_ctx* c;
  cudaStream_t s;
  cudaEvent_t b = nullptr;
  ZtmProf(ztm_ctx* ctx, const char* name, cudaStream_t stream = nullptr);
  ~ZtmProf();
};

// Fork/join of the context's side stream: work launched on c->aux between
// ztm_fork and ztm_join runs concurrently with the main stream's work and is
// ordered before everything the main stream does after the join.
void ztm_fork(ztm_ctx* c);
void ztm_join(ztm_ctx* c);

// ---------------------------------------------------------------------------
// host helpers
int ztm_fail(ztm_ctx* c, int code, const std::string& msg);
int ztm_cuda_check(ztm_ctx* c, cudaError_t e, const char* what);
// Ensure the workspace holds `bytes`; synchronises the stream before growing.
int ztm_ws_reserve(ztm_ctx* c, size_t bytes);
// Bump allocator over the workspace (256-byte aligned slices).
struct WsCarver {
  char* base;
  size_t off = 0;
  explicit WsCarver(char* b) : base(b) {}
  template <class T>
  T* take(size_t n) {
    size_t a = (off + 255) & ~size_t(255);
    off = a + n * sizeof(T);
    return reinterpret_cast<T*>(base + a);
  }
  static size_t need(size_t bytes) { return ((bytes + 255) & ~size_t(255)); }
};
// After launches: check the launch error and the device error word.
int ztm_after_launch(ztm_ctx* c, const char* what);
int ztm_check_device_error(ztm_ctx* c);

// Copy-in helper: returns device pointer for an argument (either the
// caller's device pointer or a staged copy in the workspace).
int ztm_stage_in(ztm_ctx* c, const void* src, size_t bytes, bool dev,
                 void* staged, const void** out);

// ---------------------------------------------------------------------------
// kernel launchers (implemented in the .cu files)
struct PmParams {
  int di, dj, ii, jj, kk, fh, fv, bfr;
  int ni, nj, ns;  // interior stations
  long long nnodes;  // nodes iterated (N or n_nn)
  long long N;       // fine-grid size (bounds of nn entries)
  double thr;
};
int ztm_launch_pointmass(ztm_ctx* c, const PmParams& p, const double* d_drho,
                         const int* d_nn, const double* d_surf, double* d_G,
                         double scale, int precision, WsCarver& wc);
size_t ztm_pointmass_ws(const PmParams& p, int precision, int num_sms);
// Exclusive scan of n ints in place on `s` (one block); *total = their sum.
void ztm_scan_ints(cudaStream_t s, int n, int* counts, int* total);

// Adjoint of the point-mass forward (pm_adjoint.cu): d_g[n] (all N nodes) =
// scale*66.7/(fh^2 fv) * mult(n) * sum over interior stations m of
// d_w[m] (k0-k)/r^3, where mult(n) is n's count in d_nn (p.nnodes entries)
// when d_nn is given, else 1 where |d_drho[n]| > p.thr when d_drho is given,
// else 1.  d_w has di*dj entries (the interior ones are read).
size_t ztm_pm_adjoint_ws(const PmParams& p, int precision, int num_sms, bool list);
int ztm_launch_pm_adjoint(ztm_ctx* c, const PmParams& p, const double* d_drho, const int* d_nn,
                          const double* d_surf, const double* d_w, double* d_g, double scale,
                          int precision, WsCarver& wc);
// The gravity part of TFM's misfit (TFM.cpp:101-103) from the forward's G:
// r = (GD - (G + g0)) / gsig over the bfr interior, in TFM's order (i0
// outer, j0 inner) into d_res (may be null); d_w[m] = -2 r / gsig at the
// interior stations, 0 elsewhere (the adjoint's weights for d ssq / d G);
// d_out[0] = ssq = sum r^2, d_out[1] = d ssq / d g0 = -2/gsig sum r.
size_t ztm_pm_misfit_ws(const PmParams& p);
int ztm_launch_pm_misfit(ztm_ctx* c, const PmParams& p, const double* d_G, const double* d_GD,
                         double g0, double gsig, double* d_res, double* d_w, double* d_out,
                         WsCarver& wc);
// Checks a point-mass grid and fills p (nnodes = N, every node).
int ztm_pm_setup(ztm_ctx* c, const ztm_grid* g, PmParams* p);
// End of a call: launch/device error check; in host mode copy `bytes` of
// dev_out to host_out and synchronise.
int ztm_finish(ztm_ctx* c, bool dev, void* host_out, const void* dev_out, size_t bytes,
               const char* what);

// Z-order permutation of the stations by home cell (order.cu): perm[slot]
// is the station a one-station-per-thread kernel computes in that slot.  si
// holds `stride` ints per station, the home cell's x and y first, on an
// nx x ny mesh.  Runs on `stream` (the context's stream or its side stream).
size_t ztm_station_order_ws(int ns, int nx, int ny);
int ztm_station_order(ztm_ctx* c, cudaStream_t stream, int ns, const int* si, int stride, int nx,
                      int ny, int* perm, WsCarver& wc);

struct MeshDesc {
  int nx, ny, nz;
  double x0, y0, zt, dx, dy, dz;
};
size_t ztm_prism_ws(const MeshDesc& m, int ns, int precision, int num_sms,
                    const ztm_opts* o);
int ztm_launch_prism(ztm_ctx* c, const MeshDesc& m, const double* d_rho,
                     int ns, const double* d_sxyz, double* d_gz, double G,
                     int precision, const ztm_opts* o, WsCarver& wc);
size_t ztm_prism_list_ws(long long np, int ns, int precision, int num_sms);
int ztm_launch_prism_list(ztm_ctx* c, long long np, const double* d_geom,
                          const double* d_rho, int ns, const double* d_sxyz,
                          double* d_gz, double G, int precision, double near_q,
                          WsCarver& wc);
size_t ztm_adjoint_ws(const MeshDesc& m, int ns, int precision, int num_sms, double near_q);
int ztm_launch_adjoint(ztm_ctx* c, const MeshDesc& m, int ns,
                       const double* d_sxyz, const double* d_res,
                       double* d_grho, double G, int precision,
                       const ztm_opts* o, WsCarver& wc);

struct IMeshDesc {
  int nx, ny;
  double x0, y0, dx, dy, zb;
};
size_t ztm_iface_ws(const IMeshDesc& m, int ns, int precision, int num_sms);
int ztm_launch_iface_fwd(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, int ns, const double* d_sxyz,
                         double* d_gz, double G, int precision,
                         const ztm_opts* o, WsCarver& wc);
// dgz = J_depth * vdep (the depth directional derivative of the forward)
int ztm_launch_iface_jvp(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, const double* d_vdep, int ns, const double* d_sxyz,
                         double* d_dgz, double G, int precision, const ztm_opts* o,
                         WsCarver& wc);
int ztm_launch_iface_adj(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, int ns, const double* d_sxyz,
                         const double* d_res, double* d_grho, double* d_gdep,
                         double G, int precision, const ztm_opts* o,
                         WsCarver& wc);

// ---------------------------------------------------------------------------
// device helpers
#ifdef __CUDACC__

// Closed-form corner function of the prism integral (double).
//   Phi = x ln(y+r) + y ln(x+r) - z atan(x y / (z r)),
// with the y<0 branch of ln(y+r) rewritten as ln((x^2+z^2)/(r-y)) so that
// y+r never cancels, and the 0*ln(0), z*atan limits taken as 0.
template <typename T>
__device__ __forceinline__ T ztm_xlog(T x, T y, T z, T r) {
  if (x == T(0)) return T(0);
  if (y >= T(0)) return x * log(y + r);
  return x * log((x * x + z * z) / (r - y));
}

template <typename T>
__device__ __forceinline__ T ztm_phi(T x, T y, T z) {
  T r = sqrt(x * x + y * y + z * z);
  if (r == T(0)) return T(0);
  T t = ztm_xlog(x, y, z, r) + ztm_xlog(y, x, z, r);
  if (z != T(0)) t -= z * atan(x * y / (z * r));
  return t;
}

// Integral of (zs - z)/r^3 over a prism given mass-minus-station corner
// coordinates: sum over corners of s_x s_y s_z Phi.
template <typename T>
__device__ __forceinline__ T ztm_prism_unit(T xa, T xb, T ya, T yb, T za, T zb) {
  T s = T(0);
  s -= ztm_phi(xa, ya, za);
  s += ztm_phi(xb, ya, za);
  s += ztm_phi(xa, yb, za);
  s -= ztm_phi(xb, yb, za);
  s += ztm_phi(xa, ya, zb);
  s -= ztm_phi(xb, ya, zb);
  s -= ztm_phi(xa, yb, zb);
  s += ztm_phi(xb, yb, zb);
  return s;
}

// Integral of w/r^3 over a horizontal rectangle at height w below the
// station (w = z_station - z_face), relative corners xa..xb, ya..yb.
__device__ __forceinline__ double ztm_face_unit(double xa, double xb,
                                                double ya, double yb,
                                                double w) {
  if (w == 0.0) return 0.0;
  double s = 0.0;
  double x[2] = {xa, xb}, y[2] = {ya, yb};
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      double r = sqrt(x[a] * x[a] + y[b] * y[b] + w * w);
      double t = atan(x[a] * y[b] / (w * r));
      s += (a == b) ? t : -t;
    }
  return s;
}

// Compensated (Kahan) accumulation in float.  The true sum is s - c.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const {
    return (double)s - (double)c;
  }
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ---- mbarrier + bulk copy (TMA, non-tensor) ------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
// 1-D bulk copy global -> shared, completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait on phase `parity`; returns false if `limit` spins ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          uint32_t limit = ZTM_WAIT_LIMIT) {
  uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Non-blocking test of phase `parity`, up to `limit` times; false if the phase
// was not seen complete (the timeout path's test hook).
__device__ __forceinline__ bool mbar_poll(uint64_t* bar, uint32_t parity, uint32_t limit) {
  uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

#endif  // __CUDACC__
