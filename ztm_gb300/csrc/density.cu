// density.cu - the density-perturbation builder of TFM.cpp:83-89 on the GPU.
//
// For every fine-grid node the reference interpolates the IASP91 Moho
// (sea-level map - 3.5), the rendered Moho M and the velocity field v
// (zmath.cpp:225-252), ramps the crust/mantle contrast ro across one fine
// cell around each Moho, scales the velocity perturbation by dr, and keeps
// r1 - r0 where it exceeds 0.001 g/cc at depths below 10 km (c2g, TFM.cpp:56,
// through enu2geo, SET.cpp:86-99).  Running it here leaves drho in device
// memory for ztm_gfm_pointmass (ZTM_FLAG_DEVICE_PTRS) instead of building it
// on one CPU thread and copying it in every forward.
//
// Same arithmetic as the reference, operation by operation: products and
// sums are written with __dmul_rn / __dadd_rn so that nothing is contracted
// into an FMA, the distance is taken with sqrtf as in SET.cpp:97, and the
// reference-point trigonometry (cos/sin of the reference latitude and
// longitude) is evaluated once on the host with the host's libm, as the
// reference does.  One difference: the 2-D interpolation of the reference
// reads one element past the row (or the array) at the last column/row with
// weight 0; that index is clamped here.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "ztm_internal.cuh"

namespace {

struct DensGeo {
  double m[9], xr, yr, zr, ox, oy, oz, h;
};

struct DensArgs {
  int di, dj, dk, fh, fv, ii, jj;
  long long N;
  double vm, ro, dr;
  DensGeo g;
};

__device__ __forceinline__ double lerp_rn(double a, double b, double s) {
  // a*(1-s) + b*s without contraction
  return __dadd_rn(__dmul_rn(a, __dadd_rn(1.0, -s)), __dmul_rn(b, s));
}

__device__ double interp2_dev(const double* __restrict__ f, double x, double y, int di, int dj) {
  const double ii = fmin(fmax(x, 0.0), (double)(di - 1)), jj = fmin(fmax(y, 0.0), (double)(dj - 1));
  const int i = (int)ii, j = (int)jj;
  const double si = ii - i, sj = jj - j;
  const int i1 = i + 1 < di ? i + 1 : i, j1 = j + 1 < dj ? j + 1 : j;
  const double c0 = lerp_rn(f[i + j * di], f[i1 + j * di], si);
  const double c1 = lerp_rn(f[i + j1 * di], f[i1 + j1 * di], si);
  return lerp_rn(c0, c1, sj);
}

__device__ double interp3_dev(const double* __restrict__ f, double x, double y, double z, int di,
                              int dj, int dk) {
  const double ii = fmin(fmax(x, 0.0), (double)(di - 2)), jj = fmin(fmax(y, 0.0), (double)(dj - 2)),
               kk = fmin(fmax(z, 0.0), (double)(dk - 2));
  const int i = (int)ii, j = (int)jj, k = (int)kk;
  const double si = ii - i, sj = jj - j, sk = kk - k;
  const long long p = (long long)di * dj;
  auto F = [&](int a, int b, int c) { return f[(i + a) + (long long)(j + b) * di + (k + c) * p]; };
  const double c00 = lerp_rn(F(0, 0, 0), F(1, 0, 0), si), c01 = lerp_rn(F(0, 0, 1), F(1, 0, 1), si);
  const double c10 = lerp_rn(F(0, 1, 0), F(1, 1, 0), si), c11 = lerp_rn(F(0, 1, 1), F(1, 1, 1), si);
  const double c0 = lerp_rn(c00, c10, sj), c1 = lerp_rn(c01, c11, sj);
  return lerp_rn(c0, c1, sk);
}

__device__ double depth_dev(const DensGeo& g, double i, double j, double k) {
  const double x = __dadd_rn(__dmul_rn(i, g.h), -g.ox);
  const double y = __dadd_rn(__dmul_rn(j, g.h), -g.oy);
  const double z = __dadd_rn(__dmul_rn(k, g.h), -g.oz);
  auto row = [&](int r, double o) {
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(g.m[3 * r], x), __dmul_rn(g.m[3 * r + 1], y)),
                               __dmul_rn(g.m[3 * r + 2], z)),
                     o);
  };
  const double xi = row(0, g.xr), yi = row(1, g.yr), zi = row(2, g.zr);
  const double s2 = __dadd_rn(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi)), __dmul_rn(zi, zi));
  const float r = sqrtf((float)s2);
  return 6371.0 - (double)r;
}

__device__ double ramp(double r, double k, double m, double li, double ro) {
  // if k > m+li: ro;  else if |k-m| < li: r + (k-m+li)*(r+ro)/(2*li)
  if (k > __dadd_rn(m, li)) return ro;
  const double d = __dadd_rn(k, -m);
  if (fabs(d) < li) return __dadd_rn(r, __dmul_rn(__dadd_rn(d, li), __dadd_rn(r, ro)) / (2 * li));
  return r;
}

__global__ void density_kernel(DensArgs a, const double* __restrict__ sea,
                               const double* __restrict__ M, const double* __restrict__ v,
                               double* __restrict__ drho, unsigned long long* __restrict__ count) {
  const long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool sel = false;
  if (n < a.N) {
    const double i = (n % a.ii) / (1. * a.fh), j = ((n / a.ii) % a.jj) / (1. * a.fh),
                 k = (n / ((long long)a.ii * a.jj)) / (1. * a.fv), li = 1. / a.fv;
    const double m0 = __dadd_rn(interp2_dev(sea, i, j, a.di, a.dj), -3.5);
    const double m1 = interp2_dev(M, i, j, a.di, a.dj);
    const double r0 = ramp(0.0, k, m0, li, a.ro);
    const double r1 = ramp(__dmul_rn(a.dr, __dadd_rn(interp3_dev(v, i, j, k, a.di, a.dj, a.dk), -a.vm)),
                           k, m1, li, a.ro);
    const double d = __dadd_rn(r1, -r0);
    sel = fabs(__dadd_rn(r0, -r1)) > .001 && depth_dev(a.g, i, j, k) > 10;
    drho[n] = sel ? d : 0.0;
  }
  const unsigned b = __ballot_sync(0xffffffffu, sel);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned long long)__popc(b));
}

// ---- derivative of the builder ------------------------------------------
// drho[n] = r1 - r0 (TFM.cpp:86-89) is piecewise linear in its inputs: with
// b = dr*(v(i,j,k) - vm) and t = (k - m + li)/(2 li),
//   ramp(r, k, m) = ro                     if k > m + li,
//                 = r (1 + t) + ro t       if |k - m| < li,
//                 = r                      otherwise,
// so d r1/d b, d r1/d ro, d r1/d m1 (= -(b + ro)/(2 li) in the blend) and
// d r0/d ro follow branch by branch, with the branch decided exactly as the
// forward decides it.  The node selection (|r1 - r0| > .001, depth > 10 km)
// is held fixed, as a finite-difference step that does not cross it sees.
struct RampGrad {
  double db, dro, dm;  // d ramp / d r, d ro, d m
};

__device__ RampGrad ramp_grad(double r, double k, double m, double li, double ro) {
  RampGrad g = {0.0, 0.0, 0.0};
  if (k > __dadd_rn(m, li)) {
    g.dro = 1.0;
    return g;
  }
  const double d = __dadd_rn(k, -m);
  if (fabs(d) < li) {
    const double t = __dadd_rn(d, li) / (2 * li);
    g.db = 1.0 + t;
    g.dro = t;
    g.dm = -__dadd_rn(r, ro) / (2 * li);
    return g;
  }
  g.db = 1.0;
  return g;
}

// Adds s * d interp2(f, x, y)/d f into gf (the weights of interp2_dev).
__device__ void interp2_scatter(double* __restrict__ gf, double x, double y, int di, int dj,
                                double s) {
  const double ii = fmin(fmax(x, 0.0), (double)(di - 1)), jj = fmin(fmax(y, 0.0), (double)(dj - 1));
  const int i = (int)ii, j = (int)jj;
  const double si = ii - i, sj = jj - j;
  const int i1 = i + 1 < di ? i + 1 : i, j1 = j + 1 < dj ? j + 1 : j;
  const double w[4] = {(1 - si) * (1 - sj), si * (1 - sj), (1 - si) * sj, si * sj};
  const int at[4] = {i + j * di, i1 + j * di, i + j1 * di, i1 + j1 * di};
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (w[q] != 0.0) atomicAdd(&gf[at[q]], s * w[q]);
}

// Adds s * d interp3(f, x, y, z)/d f into gf (the weights of interp3_dev).
__device__ void interp3_scatter(double* __restrict__ gf, double x, double y, double z, int di,
                                int dj, int dk, double s) {
  const double ii = fmin(fmax(x, 0.0), (double)(di - 2)), jj = fmin(fmax(y, 0.0), (double)(dj - 2)),
               kk = fmin(fmax(z, 0.0), (double)(dk - 2));
  const int i = (int)ii, j = (int)jj, k = (int)kk;
  const double si = ii - i, sj = jj - j, sk = kk - k;
  const long long pl = (long long)di * dj;
#pragma unroll
  for (int c = 0; c < 2; c++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const double w = (a ? si : 1 - si) * (b ? sj : 1 - sj) * (c ? sk : 1 - sk);
        if (w != 0.0) atomicAdd(&gf[(i + a) + (long long)(j + b) * di + (k + c) * pl], s * w);
      }
}

// From a[n] = d ssq / d drho[n] (zero off the selection): gM += d ssq / d M,
// gv += d ssq / d v (both zeroed by the caller), and per block the
// contributions to d ssq / d (vm, ro, dr).
constexpr int DENS_T = 256;
__global__ void __launch_bounds__(DENS_T)
    density_adjoint_kernel(DensArgs a, const double* __restrict__ sea,
                           const double* __restrict__ M, const double* __restrict__ v,
                           const double* __restrict__ adrho, double* __restrict__ gM,
                           double* __restrict__ gv, double* __restrict__ blk) {
  __shared__ double s_w[DENS_T / 32][3];
  const long long n = blockIdx.x * (long long)DENS_T + threadIdx.x;
  double c_vm = 0.0, c_ro = 0.0, c_dr = 0.0;
  if (n < a.N) {
    const double an = adrho[n];
    if (an != 0.0) {
      const double i = (n % a.ii) / (1. * a.fh), j = ((n / a.ii) % a.jj) / (1. * a.fh),
                   k = (n / ((long long)a.ii * a.jj)) / (1. * a.fv), li = 1. / a.fv;
      const double m0 = __dadd_rn(interp2_dev(sea, i, j, a.di, a.dj), -3.5);
      const double m1 = interp2_dev(M, i, j, a.di, a.dj);
      const double vi = interp3_dev(v, i, j, k, a.di, a.dj, a.dk);
      const double b = __dmul_rn(a.dr, __dadd_rn(vi, -a.vm));
      const RampGrad g0 = ramp_grad(0.0, k, m0, li, a.ro);
      const RampGrad g1 = ramp_grad(b, k, m1, li, a.ro);
      // drho = r1 - r0
      if (g1.db != 0.0) interp3_scatter(gv, i, j, k, a.di, a.dj, a.dk, an * g1.db * a.dr);
      if (g1.dm != 0.0) interp2_scatter(gM, i, j, a.di, a.dj, an * g1.dm);
      c_vm = -an * g1.db * a.dr;
      c_dr = an * g1.db * (vi - a.vm);
      c_ro = an * (g1.dro - g0.dro);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c_vm += __shfl_down_sync(0xffffffffu, c_vm, o);
    c_ro += __shfl_down_sync(0xffffffffu, c_ro, o);
    c_dr += __shfl_down_sync(0xffffffffu, c_dr, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_w[threadIdx.x >> 5][0] = c_vm;
    s_w[threadIdx.x >> 5][1] = c_ro;
    s_w[threadIdx.x >> 5][2] = c_dr;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int q = 0; q < DENS_T / 32; q++) t += s_w[q][threadIdx.x];
    blk[blockIdx.x * 3LL + threadIdx.x] = t;
  }
}

// out[c] = sum over blocks of blk[b*3 + c], in block order (one warp each).
__global__ void density_adjoint_total(long long nblk, const double* __restrict__ blk,
                                      double* __restrict__ out) {
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (c >= 3) return;
  double t = 0.0;
  for (long long b = lane; b < nblk; b += 32) t += blk[b * 3 + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if (lane == 0) out[c] = t;
}

// Checks the parameters and fills the kernel arguments.
int dens_setup(ztm_ctx* c, const ztm_density_params* p, DensArgs* a) {
  if (p->di < 2 || p->dj < 2 || p->dk < 2 || p->fh < 1 || p->fv < 1)
    return ztm_fail(c, ZTM_ERR_ARG, "grid dims must be >= 2 and refinements >= 1");
  a->di = p->di; a->dj = p->dj; a->dk = p->dk; a->fh = p->fh; a->fv = p->fv;
  a->ii = (p->di - 1) * p->fh + 1;
  a->jj = (p->dj - 1) * p->fh + 1;
  a->N = (long long)a->ii * a->jj * ((p->dk - 1) * p->fv + 1);
  if (a->N > (1LL << 31) - 1) return ztm_fail(c, ZTM_ERR_RANGE, "fine grid exceeds 2^31-1 nodes");
  a->vm = p->vm; a->ro = p->ro; a->dr = p->dr;
  // enu2geo's reference-point terms (SET.cpp:87-93), host libm as in the reference
  const double rad = 57.295, R = 6371;
  const double* rc = p->rc;
  const double phi = rc[0] / rad, theta = rc[1] / rad;
  const double m[9] = {-sin(theta), -sin(phi) * cos(theta), cos(phi) * cos(theta),
                       cos(theta),  -sin(phi) * sin(theta), cos(phi) * sin(theta),
                       0,           cos(phi),               sin(phi)};
  for (int t = 0; t < 9; t++) a->g.m[t] = m[t];
  a->g.xr = (R - rc[2]) * cos(rc[1] / rad) * cos(rc[0] / rad);
  a->g.yr = (R - rc[2]) * sin(rc[1] / rad) * cos(rc[0] / rad);
  a->g.zr = (R - rc[2]) * sin(rc[0] / rad);
  a->g.ox = rc[3]; a->g.oy = rc[4]; a->g.oz = rc[5]; a->g.h = rc[6];
  return ZTM_OK;
}

struct DevRestore {
  int p = -1, d;
  explicit DevRestore(int dev) : d(dev) {
    cudaGetDevice(&p);
    if (p != d) cudaSetDevice(d);
  }
  ~DevRestore() {
    if (p >= 0 && p != d) cudaSetDevice(p);
  }
};

// Stages sea, M, v and launches the builder into `out` (device).
int dens_run(ztm_ctx* c, const DensArgs& a, const double* sea, const double* M, const double* v,
             bool dev, WsCarver& wc, double* out, unsigned long long* cnt) {
  const size_t M2 = (size_t)a.di * a.dj, M3 = M2 * a.dk;
  double* s_sea = wc.take<double>(M2);
  double* s_M = wc.take<double>(M2);
  double* s_v = wc.take<double>(M3);
  const void *ps, *pm, *pv;
  int rc;
  if ((rc = ztm_stage_in(c, sea, M2 * 8, dev, s_sea, &ps))) return rc;
  if ((rc = ztm_stage_in(c, M, M2 * 8, dev, s_M, &pm))) return rc;
  if ((rc = ztm_stage_in(c, v, M3 * 8, dev, s_v, &pv))) return rc;
  cudaMemsetAsync(cnt, 0, 8, c->stream);
  {
    ZtmProf prof_(c, "density");
    density_kernel<<<(unsigned)((a.N + 255) / 256), 256, 0, c->stream>>>(
        a, (const double*)ps, (const double*)pm, (const double*)pv, out, cnt);
  }
  c->launches++;
  return ztm_after_launch(c, "density builder");
}

size_t dens_ws(const DensArgs& a) {
  const size_t M2 = (size_t)a.di * a.dj, M3 = M2 * a.dk;
  return 2 * WsCarver::need(M2 * 8) + WsCarver::need(M3 * 8) + WsCarver::need(8);
}

}  // namespace

extern "C" int ztm_density_build(ztm_ctx* c, const ztm_density_params* p, const double* sea,
                                 const double* M, const double* v, double* drho,
                                 long long* n_selected, int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!p || !sea || !M || !v || !drho) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  DensArgs a;
  int rc2 = dens_setup(c, p, &a);
  if (rc2) return rc2;
  DevRestore restore(c->device);
  size_t need = dens_ws(a) + WsCarver::need(a.N * 8) + 4096;
  if ((rc2 = ztm_ws_reserve(c, need))) return rc2;
  WsCarver wc(c->ws);
  double* s_d = wc.take<double>(a.N);
  unsigned long long* cnt = wc.take<unsigned long long>(1);
  double* out = dev ? drho : s_d;
  if ((rc2 = dens_run(c, a, sea, M, v, dev, wc, out, cnt))) return rc2;
  if (!dev) {
    unsigned long long h = 0;
    cudaMemcpyAsync(drho, s_d, a.N * 8, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, c->stream);
    if ((rc2 = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "density builder"))) return rc2;
    if (n_selected) *n_selected = (long long)h;
  } else if (n_selected) {
    *n_selected = -1;  // not waited for with device pointers
  }
  return ZTM_OK;
}

// TFM.cpp:83-99 in one call: the builder writes drho into the workspace and
// the point-mass forward reads it there (nodes with |drho| > threshold; the
// builder has zeroed every node TFM.cpp:89 leaves out of nn).
extern "C" int ztm_gfm_pointmass_model(ztm_ctx* c, const ztm_density_params* dp,
                                       const ztm_grid* g, const double* sea, const double* M,
                                       const double* v, const double* surf, double* G,
                                       int precision, int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!dp || !g || !sea || !M || !v || !surf || !G)
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32)
    return ztm_fail(c, ZTM_ERR_ARG, "point-mass precision must be FP64 or FP32");
  if (dp->di != g->di || dp->dj != g->dj || dp->dk != g->dk || dp->fh != g->fh || dp->fv != g->fv)
    return ztm_fail(c, ZTM_ERR_ARG, "density and grid dimensions differ");
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  DensArgs a;
  int rc = dens_setup(c, dp, &a);
  if (rc) return rc;
  PmParams p;
  if ((rc = ztm_pm_setup(c, g, &p))) return rc;
  DevRestore restore(c->device);
  const size_t M2 = (size_t)g->di * g->dj;
  size_t need = dens_ws(a) + WsCarver::need(a.N * 8) + 2 * WsCarver::need(M2 * 8) +
                ztm_pointmass_ws(p, precision, c->num_sms) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* d_rho = wc.take<double>(a.N);
  unsigned long long* cnt = wc.take<unsigned long long>(1);
  double* s_surf = wc.take<double>(M2);
  double* s_G = wc.take<double>(M2);
  if ((rc = dens_run(c, a, sea, M, v, dev, wc, d_rho, cnt))) return rc;
  const void* ps;
  if ((rc = ztm_stage_in(c, surf, M2 * 8, dev, s_surf, &ps))) return rc;
  double* outG = dev ? G : s_G;
  rc = ztm_launch_pointmass(c, p, d_rho, nullptr, (const double*)ps, outG, g->scale, precision, wc);
  if (rc) return rc;
  return ztm_finish(c, dev, G, outG, M2 * 8, "density + point-mass forward");
}

// TFM.cpp:83-103 with its derivative: the builder, the point-mass forward
// over the nodes it selects, the gravity misfit of TFM.cpp:101-103, and (when
// a gradient is asked for) the transposed point-mass sum chained back through
// the builder to the rendered Moho M, the velocity grid v and (vm, ro, dr),
// plus d ssq / d g0.  Replaces the gravity columns of the finite-difference
// Jacobian of TFM.cpp:124-135 (one forward per parameter) by one forward and
// one adjoint.
extern "C" int ztm_gfm_pointmass_model_misfit(ztm_ctx* c, const ztm_density_params* dp,
                                              const ztm_grid* g, const double* sea,
                                              const double* M, const double* v, const double* surf,
                                              const double* GD, double g0, double gsig,
                                              double* ssq, double* res, double* G, double* g_M,
                                              double* g_v, double* g_par, int precision,
                                              int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!dp || !g || !sea || !M || !v || !surf || !GD || !ssq)
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32)
    return ztm_fail(c, ZTM_ERR_ARG, "point-mass precision must be FP64 or FP32");
  if (dp->di != g->di || dp->dj != g->dj || dp->dk != g->dk || dp->fh != g->fh || dp->fv != g->fv)
    return ztm_fail(c, ZTM_ERR_ARG, "density and grid dimensions differ");
  if (!(gsig > 0) || !isfinite(g0)) return ztm_fail(c, ZTM_ERR_ARG, "gsig must be > 0, g0 finite");
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  const bool grad = g_M || g_v || g_par;
  DensArgs a;
  int rc = dens_setup(c, dp, &a);
  if (rc) return rc;
  PmParams p;
  if ((rc = ztm_pm_setup(c, g, &p))) return rc;
  DevRestore restore(c->device);
  const size_t M2 = (size_t)g->di * g->dj, M3 = M2 * g->dk;
  const long long nblk = (a.N + DENS_T - 1) / DENS_T;
  size_t need = dens_ws(a) + WsCarver::need(a.N * 8) + WsCarver::need(8) +
                4 * WsCarver::need(M2 * 8) + WsCarver::need((size_t)std::max(p.ns, 1) * 8) +
                WsCarver::need(16) + WsCarver::need(a.N * 8) + WsCarver::need(M2 * 8) +
                WsCarver::need(M3 * 8) + WsCarver::need((size_t)nblk * 24) + WsCarver::need(32) +
                ztm_pm_misfit_ws(p) +
                std::max(ztm_pointmass_ws(p, precision, c->num_sms),
                         grad ? ztm_pm_adjoint_ws(p, precision, c->num_sms, false) : 0) +
                4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* d_rho = wc.take<double>(a.N);
  unsigned long long* cnt = wc.take<unsigned long long>(1);
  double* s_surf = wc.take<double>(M2);
  double* s_GD = wc.take<double>(M2);
  double* s_G = wc.take<double>(M2);
  double* s_w = wc.take<double>(M2);
  double* s_res = wc.take<double>((size_t)std::max(p.ns, 1));
  double* s_out = wc.take<double>(2);
  double* s_a = wc.take<double>(a.N);
  double* s_gM = wc.take<double>(M2);
  double* s_gv = wc.take<double>(M3);
  double* s_blk = wc.take<double>((size_t)nblk * 3);
  double* s_par = wc.take<double>(4);
  // dens_run stages sea, M and v in the first three slices of its carver;
  // they stay there for the builder's adjoint
  WsCarver dw = wc, q = wc;
  const double* a_sea = q.take<double>(M2);
  const double* a_M = q.take<double>(M2);
  const double* a_v = q.take<double>(M3);
  if ((rc = dens_run(c, a, sea, M, v, dev, dw, d_rho, cnt))) return rc;
  const double* pse = dev ? sea : a_sea;
  const double* pM = dev ? M : a_M;
  const double* pv = dev ? v : a_v;
  WsCarver after = dw;  // past the staged sea, M, v
  const void *ps, *pgd;
  if ((rc = ztm_stage_in(c, surf, M2 * 8, dev, s_surf, &ps))) return rc;
  if ((rc = ztm_stage_in(c, GD, M2 * 8, dev, s_GD, &pgd))) return rc;
  double* oG = (dev && G) ? G : s_G;
  double* ores = res ? (dev ? res : s_res) : nullptr;
  {
    WsCarver t = after;
    rc = ztm_launch_pointmass(c, p, d_rho, nullptr, (const double*)ps, oG, g->scale, precision, t);
    if (rc) return rc;
  }
  WsCarver t2 = after;
  rc = ztm_launch_pm_misfit(c, p, oG, (const double*)pgd, g0, gsig, ores, s_w, s_out, t2);
  if (rc) return rc;
  if (grad) {
    WsCarver t3 = t2;
    rc = ztm_launch_pm_adjoint(c, p, d_rho, nullptr, (const double*)ps, s_w, s_a, g->scale,
                               precision, t3);
    if (rc) return rc;
    double* ogM = (dev && g_M) ? g_M : s_gM;
    double* ogv = (dev && g_v) ? g_v : s_gv;
    cudaMemsetAsync(ogM, 0, M2 * 8, c->stream);
    cudaMemsetAsync(ogv, 0, M3 * 8, c->stream);
    density_adjoint_kernel<<<(unsigned)nblk, DENS_T, 0, c->stream>>>(a, pse, pM, pv, s_a, ogM, ogv,
                                                                     s_blk);
    density_adjoint_total<<<1, 96, 0, c->stream>>>(nblk, s_blk, s_par);
    cudaMemcpyAsync(s_par + 3, s_out + 1, 8, cudaMemcpyDeviceToDevice, c->stream);
    c->launches += 2;
    if (dev && g_par) cudaMemcpyAsync(g_par, s_par, 32, cudaMemcpyDeviceToDevice, c->stream);
    if (!dev) {
      if (g_M) cudaMemcpyAsync(g_M, ogM, M2 * 8, cudaMemcpyDeviceToHost, c->stream);
      if (g_v) cudaMemcpyAsync(g_v, ogv, M3 * 8, cudaMemcpyDeviceToHost, c->stream);
      if (g_par) cudaMemcpyAsync(g_par, s_par, 32, cudaMemcpyDeviceToHost, c->stream);
    }
  }
  if (dev) {
    cudaMemcpyAsync(ssq, s_out, 8, cudaMemcpyDeviceToDevice, c->stream);
    return ztm_finish(c, true, nullptr, nullptr, 0, "density + point-mass misfit");
  }
  double h = 0.0;
  cudaMemcpyAsync(&h, s_out, 8, cudaMemcpyDeviceToHost, c->stream);
  if (G) cudaMemcpyAsync(G, oG, M2 * 8, cudaMemcpyDeviceToHost, c->stream);
  if (res && p.ns > 0)
    cudaMemcpyAsync(res, ores, (size_t)p.ns * 8, cudaMemcpyDeviceToHost, c->stream);
  rc = ztm_finish(c, false, nullptr, nullptr, 0, "density + point-mass misfit");
  if (rc) return rc;
  *ssq = h;
  return ZTM_OK;
}
