// pm_adjoint.cu - the transposed point-mass sum and the reference-form misfit.
//
// The reference optimiser differentiates its gravity model by forward
// differences of whole forward runs (TFM.cpp:124-135: one FM call per
// parameter).  The derivative of the point-mass field of TFM.cpp:96-98,
//     G[m] = c * sum_n drho[n] (k0_m - k_n) / r_mn^3,   c = 66.7/(fh^2 fv),
// with respect to the density of node n is c (k0_m - k_n) / r_mn^3, so one
// pass of the transposed sum
//     g[n] = c * sum_m w[m] (k0_m - k_n) / r_mn^3
// gives J^T w for any station weights w, in particular the gradient of the
// gravity misfit of TFM.cpp:101-103 (w = -2 r / gsig).
//
// Layout.  A node column (fine-grid column c = i + j*ii) shares its horizontal
// offset to a station, so a thread owns a group of LV selected levels of one
// column and forms X^2 + Y^2 once per station for all of them; the interior
// stations stream through shared memory tile by tile (one broadcast read per
// station).  The groups are built once per call: pma_count (groups per
// column), a scan, pma_write (the group's column and levels).  Float groups
// hold 8 levels as 4 packed pairs (FADD2/FFMA2/FMUL2, the rsqrt on the SFU),
// with plain float sums over 32 stations and Kahan sums across; double groups
// hold 4 levels.  grid.y splits the stations into slices whose partial sums
// pma_finalize adds in a fixed order: no atomics, bitwise reproducible.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "ztm_internal.cuh"

namespace {

constexpr int PMA_TB = 128;  // groups (threads) per block
constexpr int PMA_ST = 256;  // stations per shared-memory tile

template <bool F64>
struct PmaT;
template <>
struct PmaT<false> {
  static constexpr int LV = 8;  // levels per group
  using S = float4;             // station (i0, j0, k0, w)
};
template <>
struct PmaT<true> {
  static constexpr int LV = 4;
  struct __align__(16) S {
    double x, y, z, w;
  };
};

__device__ __forceinline__ float pma_rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Node multiplicities of a list (a node listed twice counts twice, as in the
// reference loop TFM.cpp:97); entries outside the grid are recorded.
__global__ void pma_mark(long long nlist, long long N, const int* __restrict__ nn,
                         int* __restrict__ mult, int* __restrict__ err) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nlist) return;
  const long long n = nn[t];
  if (n < 0 || n >= N) {
    atomicOr(err, ZTM_DEVERR_BOUNDS);
    return;
  }
  atomicAdd(&mult[n], 1);
}

// Selection factor of node n: its multiplicity (list), 1 or 0 by the
// threshold (densities), or 1 (every node).
__device__ __forceinline__ int pma_sel(const PmParams& p, const int* __restrict__ mult,
                                       const double* __restrict__ drho, long long n) {
  if (mult) return mult[n];
  if (drho) return fabs(drho[n]) > p.thr ? 1 : 0;
  return 1;
}

template <int LV>
__global__ void pma_count(PmParams p, const int* __restrict__ mult,
                          const double* __restrict__ drho, int* __restrict__ counts) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  int cnt = 0;
  for (int k = 0; k < p.kk; k++)
    if (pma_sel(p, mult, drho, c + k * ncols)) cnt++;
  counts[c] = (cnt + LV - 1) / LV;
}

// Groups of column c: gcol[g] = c, glev[g*LV + l] = level (or -1 past the
// column's last selected level).
template <int LV>
__global__ void pma_write(PmParams p, const int* __restrict__ mult, const double* __restrict__ drho,
                          const int* __restrict__ offs, int* __restrict__ gcol,
                          short* __restrict__ glev) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  int g = offs[c], l = 0;
  for (int k = 0; k < p.kk; k++) {
    if (!pma_sel(p, mult, drho, c + k * ncols)) continue;
    if (l == 0) gcol[g] = (int)c;
    glev[(long long)g * LV + l] = (short)k;
    if (++l == LV) {
      l = 0;
      g++;
    }
  }
  if (l) {
    for (; l < LV; l++) glev[(long long)g * LV + l] = -1;
  }
}

// Interior stations in interior order s = (i0-bfr) + (j0-bfr)*ni, with their
// weights; slots past ns are zero weights far away.
template <bool F64>
__global__ void pma_stations(PmParams p, const double* __restrict__ surf,
                             const double* __restrict__ w, int nslots,
                             typename PmaT<F64>::S* __restrict__ st) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  typename PmaT<F64>::S v;
  if (s < p.ns) {
    const int i0 = p.bfr + s % p.ni, j0 = p.bfr + s / p.ni, m = i0 + j0 * p.di;
    v.x = i0;
    v.y = j0;
    v.z = surf[m];  // float groups: the height travels as float, as in the forward
    v.w = w[m];
  } else {
    v.x = 1.0e18f;
    v.y = 1.0e18f;
    v.z = 0;
    v.w = 0;
  }
  st[s] = v;
}

// Float groups: 8 levels of one column per thread, 4 packed pairs.
__global__ void __launch_bounds__(PMA_TB)
    pma_gather_f32(PmParams p, const int* __restrict__ n_groups, const int* __restrict__ gcol,
                   const short* __restrict__ glev, const float4* __restrict__ st, int slice_len,
                   long long pstride, double* __restrict__ partial) {
  __shared__ float4 tile[PMA_ST];
  const int ng = *n_groups;
  const int g = blockIdx.x * PMA_TB + threadIdx.x;
  const bool active = g < ng;
  float nx = 0.f, ny = 0.f;
  float2 kz[4];
#pragma unroll
  for (int q = 0; q < 4; q++) kz[q] = make_float2(-1.0e18f, -1.0e18f);
  if (active) {
    const int c = gcol[g];
    nx = -(float)((c % p.ii) * (1.0 / p.fh));  // -i, -j in grid units (TFM.cpp:97)
    ny = -(float)((c / p.ii) * (1.0 / p.fh));
    const short4 a = reinterpret_cast<const short4*>(glev)[2 * (long long)g];
    const short4 b = reinterpret_cast<const short4*>(glev)[2 * (long long)g + 1];
    const short lv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      kz[q].x = lv[2 * q] >= 0 ? -(float)(lv[2 * q] * (1.0 / p.fv)) : -1.0e18f;
      kz[q].y = lv[2 * q + 1] >= 0 ? -(float)(lv[2 * q + 1] * (1.0 / p.fv)) : -1.0e18f;
    }
  }
  const int s0 = blockIdx.y * slice_len;
  const int s1 = s0 + slice_len;  // slots past ns are zero weights
  Kahan acc[8];
  for (int t0 = s0; t0 < s1; t0 += PMA_ST) {
    __syncthreads();  // the previous tile is consumed
    for (int q = threadIdx.x; q < PMA_ST; q += PMA_TB) tile[q] = st[t0 + q];
    __syncthreads();
    if (!active) continue;
    for (int q0 = 0; q0 < PMA_ST; q0 += 32) {
      float2 gs[4];
#pragma unroll
      for (int q = 0; q < 4; q++) gs[q] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int q = q0; q < q0 + 32; q++) {
        const float4 s = tile[q];  // (i0, j0, k0, w)
        const float X = s.x + nx, Y = s.y + ny;
        const float h = fmaf(X, X, Y * Y);
        const float2 h2 = make_float2(h, h), K0 = make_float2(s.z, s.z), W = make_float2(s.w, s.w);
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const float2 dz = __fadd2_rn(K0, kz[r]);
          const float2 d2 = __ffma2_rn(dz, dz, h2);
          const float2 rs = make_float2(pma_rsqrt_ftz(d2.x), pma_rsqrt_ftz(d2.y));
          const float2 tw = __fmul2_rn(W, dz);
          gs[r] = __ffma2_rn(__fmul2_rn(tw, __fmul2_rn(rs, rs)), rs, gs[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < 4; r++) {
        acc[2 * r].add(gs[r].x);
        acc[2 * r + 1].add(gs[r].y);
      }
    }
  }
  if (active) {
    double* out = partial + blockIdx.y * pstride + (long long)g * 8;
#pragma unroll
    for (int l = 0; l < 8; l++) out[l] = acc[l].value();
  }
}

// Double groups: 4 levels of one column per thread.
__global__ void __launch_bounds__(PMA_TB)
    pma_gather_f64(PmParams p, const int* __restrict__ n_groups, const int* __restrict__ gcol,
                   const short* __restrict__ glev, const PmaT<true>::S* __restrict__ st,
                   int slice_len, long long pstride, double* __restrict__ partial) {
  __shared__ PmaT<true>::S tile[PMA_ST];
  const int ng = *n_groups;
  const int g = blockIdx.x * PMA_TB + threadIdx.x;
  const bool active = g < ng;
  double nx = 0.0, ny = 0.0, kz[4] = {-1.0e18, -1.0e18, -1.0e18, -1.0e18};
  if (active) {
    const int c = gcol[g];
    nx = -((c % p.ii) * (1.0 / p.fh));
    ny = -((c / p.ii) * (1.0 / p.fh));
    const short4 a = reinterpret_cast<const short4*>(glev)[g];
    const short lv[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int q = 0; q < 4; q++) kz[q] = lv[q] >= 0 ? -(lv[q] * (1.0 / p.fv)) : -1.0e18;
  }
  const int s0 = blockIdx.y * slice_len;
  const int s1 = s0 + slice_len;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int t0 = s0; t0 < s1; t0 += PMA_ST) {
    __syncthreads();
    for (int q = threadIdx.x; q < PMA_ST; q += PMA_TB) tile[q] = st[t0 + q];
    __syncthreads();
    if (!active) continue;
#pragma unroll 2
    for (int q = 0; q < PMA_ST; q++) {
      const PmaT<true>::S s = tile[q];
      const double X = s.x + nx, Y = s.y + ny;
      const double h = X * X + Y * Y;
#pragma unroll
      for (int r = 0; r < 4; r++) {
        const double dz = s.z + kz[r];
        const double rs = rsqrt(dz * dz + h);
        acc[r] += s.w * dz * (rs * rs * rs);
      }
    }
  }
  if (active) {
    double* out = partial + blockIdx.y * pstride + (long long)g * 4;
#pragma unroll
    for (int l = 0; l < 4; l++) out[l] = acc[l];
  }
}

// g[col + k*ncols] = factor * sel(n) * sum over slices, for every group level.
template <int LV>
__global__ void pma_finalize(PmParams p, const int* __restrict__ n_groups,
                             const int* __restrict__ gcol, const short* __restrict__ glev,
                             const int* __restrict__ mult, const double* __restrict__ drho,
                             const double* __restrict__ partial, int nslices, long long pstride,
                             double factor, double* __restrict__ out) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)*n_groups * LV) return;
  const int k = glev[t];
  if (k < 0) return;
  const long long ncols = (long long)p.ii * p.jj;
  const long long n = gcol[t / LV] + k * ncols;
  double v = 0.0;
  for (int sl = 0; sl < nslices; sl++) v += partial[sl * pstride + t];
  out[n] = factor * pma_sel(p, mult, drho, n) * v;
}

// ---- misfit --------------------------------------------------------------
constexpr int PMM_T = 256;

// Residuals in TFM's order (TFM.cpp:102: i0 outer, j0 inner) and the
// adjoint's station weights; per-block sums of r^2 and r.
__global__ void __launch_bounds__(PMM_T)
    pm_misfit_kernel(PmParams p, const double* __restrict__ G, const double* __restrict__ GD,
                     double g0, double gsig, double* __restrict__ res, double* __restrict__ w,
                     double2* __restrict__ blk) {
  __shared__ double2 s_w[PMM_T / 32];
  const int t = blockIdx.x * PMM_T + threadIdx.x;
  double r = 0.0;
  if (t < p.ns) {
    const int i0 = p.bfr + t / p.nj, j0 = p.bfr + t % p.nj, m = i0 + j0 * p.di;
    // y = GD/gsig, f = (G + g0)/gsig, res = y - f (TFM.cpp:102-103)
    r = GD[m] / gsig - (G[m] + g0) / gsig;
    if (res) res[t] = r;
    w[m] = -2.0 * r / gsig;
  }
  double2 v = make_double2(r * r, r);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 b = make_double2(0.0, 0.0);
    for (int q = 0; q < PMM_T / 32; q++) {
      b.x += s_w[q].x;
      b.y += s_w[q].y;
    }
    blk[blockIdx.x] = b;
  }
}

// out[0] = sum r^2, out[1] = -2/gsig sum r, from the block sums in order.
__global__ void pm_misfit_total(int nblk, const double2* __restrict__ blk, double gsig,
                                double* __restrict__ out) {
  __shared__ double2 s_w[32];
  double2 v = make_double2(0.0, 0.0);
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    v.x += blk[b].x;
    v.y += blk[b].y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 b = make_double2(0.0, 0.0);
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
      b.x += s_w[q].x;
      b.y += s_w[q].y;
    }
    out[0] = b.x;
    out[1] = -2.0 * b.y / gsig;
  }
}

int pma_occupancy(bool f64) {
  int occ = 0;
  cudaError_t e = f64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pma_gather_f64, PMA_TB, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pma_gather_f32, PMA_TB, 0);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    occ = 1;
  }
  return occ;
}

struct PmaShape {
  long long max_groups;  // upper bound of the groups (every column full)
  int blocks, slices, slice_len, nslots;
};

// Group blocks x station slices: about four waves of resident blocks, slices
// of whole tiles.
PmaShape pma_shape(const PmParams& p, bool f64, int num_sms) {
  PmaShape s;
  const int LV = f64 ? PmaT<true>::LV : PmaT<false>::LV;
  s.max_groups = std::max(1LL, (long long)p.ii * p.jj * ((p.kk + LV - 1) / LV));
  s.blocks = (int)((s.max_groups + PMA_TB - 1) / PMA_TB);
  const int tiles = std::max(1, (p.ns + PMA_ST - 1) / PMA_ST);
  const long long want = (4LL * pma_occupancy(f64) * std::max(num_sms, 1) + s.blocks - 1) / s.blocks;
  s.slices = (int)std::max(1LL, std::min<long long>(std::min<long long>(want, tiles), 65535));
  const int tps = (tiles + s.slices - 1) / s.slices;  // tiles per slice
  s.slice_len = tps * PMA_ST;
  s.slices = (tiles + tps - 1) / tps;
  s.nslots = s.slices * s.slice_len;
  return s;
}

}  // namespace

size_t ztm_pm_adjoint_ws(const PmParams& p, int precision, int num_sms, bool list) {
  const bool f64 = precision == ZTM_PREC_FP64;
  const PmaShape s = pma_shape(p, f64, num_sms);
  const int LV = f64 ? PmaT<true>::LV : PmaT<false>::LV;
  const long long ncols = (long long)p.ii * p.jj;
  return WsCarver::need((size_t)(ncols + 1) * sizeof(int)) +
         WsCarver::need((size_t)s.max_groups * sizeof(int)) +
         WsCarver::need((size_t)s.max_groups * LV * sizeof(short)) +
         WsCarver::need((size_t)s.nslots * (f64 ? 32 : 16)) +
         WsCarver::need((size_t)s.slices * s.max_groups * LV * sizeof(double)) +
         (list ? WsCarver::need((size_t)p.N * sizeof(int)) : 0);
}

int ztm_launch_pm_adjoint(ztm_ctx* c, const PmParams& p, const double* d_drho, const int* d_nn,
                          const double* d_surf, const double* d_w, double* d_g, double scale,
                          int precision, WsCarver& wc) {
  const bool f64 = precision == ZTM_PREC_FP64;
  const PmaShape s = pma_shape(p, f64, c->num_sms);
  const int LV = f64 ? PmaT<true>::LV : PmaT<false>::LV;
  const long long ncols = (long long)p.ii * p.jj;
  int* offs = wc.take<int>((size_t)ncols + 1);
  int* gcol = wc.take<int>((size_t)s.max_groups);
  short* glev = wc.take<short>((size_t)s.max_groups * LV);
  void* st = wc.take<char>((size_t)s.nslots * (f64 ? 32 : 16));
  double* partial = wc.take<double>((size_t)s.slices * s.max_groups * LV);
  int* mult = nullptr;
  cudaMemsetAsync(d_g, 0, (size_t)p.N * sizeof(double), c->stream);
  if (p.ns == 0 || p.nnodes == 0) return ztm_after_launch(c, "point-mass adjoint");
  if (d_nn) {
    mult = wc.take<int>((size_t)p.N);
    cudaMemsetAsync(mult, 0, (size_t)p.N * sizeof(int), c->stream);
    pma_mark<<<(unsigned)((p.nnodes + 255) / 256), 256, 0, c->stream>>>(p.nnodes, p.N, d_nn, mult,
                                                                        c->d_err);
    c->launches++;
    d_drho = nullptr;
  }
  const unsigned cb = (unsigned)((ncols + 255) / 256);
  const unsigned sb = (unsigned)((s.nslots + 255) / 256);
  const long long pstride = s.max_groups * LV;
  const double factor = scale * 66.7 / ((double)p.fh * p.fh * p.fv);
  dim3 grid(s.blocks, s.slices);
  if (f64) {
    pma_count<4><<<cb, 256, 0, c->stream>>>(p, mult, d_drho, offs);
    ztm_scan_ints(c->stream, (int)ncols, offs, offs + ncols);
    pma_write<4><<<cb, 256, 0, c->stream>>>(p, mult, d_drho, offs, gcol, glev);
    auto* sv = static_cast<PmaT<true>::S*>(st);
    pma_stations<true><<<sb, 256, 0, c->stream>>>(p, d_surf, d_w, s.nslots, sv);
    {
      ZtmProf prof_(c, "pointmass_adjoint");
      pma_gather_f64<<<grid, PMA_TB, 0, c->stream>>>(p, offs + ncols, gcol, glev, sv, s.slice_len,
                                                     pstride, partial);
    }
    pma_finalize<4><<<(unsigned)((pstride + 255) / 256), 256, 0, c->stream>>>(
        p, offs + ncols, gcol, glev, mult, d_drho, partial, s.slices, pstride, factor, d_g);
  } else {
    pma_count<8><<<cb, 256, 0, c->stream>>>(p, mult, d_drho, offs);
    ztm_scan_ints(c->stream, (int)ncols, offs, offs + ncols);
    pma_write<8><<<cb, 256, 0, c->stream>>>(p, mult, d_drho, offs, gcol, glev);
    auto* sv = static_cast<float4*>(st);
    pma_stations<false><<<sb, 256, 0, c->stream>>>(p, d_surf, d_w, s.nslots, sv);
    {
      ZtmProf prof_(c, "pointmass_adjoint");
      pma_gather_f32<<<grid, PMA_TB, 0, c->stream>>>(p, offs + ncols, gcol, glev, sv, s.slice_len,
                                                     pstride, partial);
    }
    pma_finalize<8><<<(unsigned)((pstride + 255) / 256), 256, 0, c->stream>>>(
        p, offs + ncols, gcol, glev, mult, d_drho, partial, s.slices, pstride, factor, d_g);
  }
  c->launches += 6;
  return ztm_after_launch(c, "point-mass adjoint");
}

size_t ztm_pm_misfit_ws(const PmParams& p) {
  const int nblk = std::max(1, (p.ns + PMM_T - 1) / PMM_T);
  return WsCarver::need((size_t)nblk * sizeof(double2));
}

int ztm_launch_pm_misfit(ztm_ctx* c, const PmParams& p, const double* d_G, const double* d_GD,
                         double g0, double gsig, double* d_res, double* d_w, double* d_out,
                         WsCarver& wc) {
  const int nblk = std::max(1, (p.ns + PMM_T - 1) / PMM_T);
  double2* blk = wc.take<double2>((size_t)nblk);
  cudaMemsetAsync(d_w, 0, (size_t)p.di * p.dj * sizeof(double), c->stream);
  pm_misfit_kernel<<<nblk, PMM_T, 0, c->stream>>>(p, d_G, d_GD, g0, gsig, d_res, d_w, blk);
  pm_misfit_total<<<1, 256, 0, c->stream>>>(nblk, blk, gsig, d_out);
  c->launches += 2;
  return ztm_after_launch(c, "point-mass misfit");
}

// ---------------------------------------------------------------------------
// C ABI
namespace {
struct DevGuard {
  int prev = -1;
  bool ok = true;
  explicit DevGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = (cudaSetDevice(dev) == cudaSuccess);
  }
  ~DevGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

int check_nn_host(ztm_ctx* c, const int* nn, long long n_nn, long long N, bool dev) {
  if (nn && n_nn < 0) return ztm_fail(c, ZTM_ERR_ARG, "n_nn < 0");
  if (nn && !dev)
    for (long long t = 0; t < n_nn; t++)
      if (nn[t] < 0 || nn[t] >= N)
        return ztm_fail(c, ZTM_ERR_RANGE, "nn[" + std::to_string(t) + "] outside the fine grid");
  return ZTM_OK;
}
}  // namespace

extern "C" int ztm_gfm_pointmass_adjoint(ztm_ctx* c, const ztm_grid* g, const double* drho,
                                         const int* nn, long long n_nn, const double* surf,
                                         const double* w, double* g_drho, int precision,
                                         int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!g || !surf || !w || !g_drho) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32)
    return ztm_fail(c, ZTM_ERR_ARG, "point-mass precision must be FP64 or FP32");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  PmParams p;
  int rc = ztm_pm_setup(c, g, &p);
  if (rc) return rc;
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  if ((rc = check_nn_host(c, nn, n_nn, p.N, dev))) return rc;
  if (nn) p.nnodes = n_nn;
  const long long M = (long long)g->di * g->dj;
  DevGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  const bool use_rho = !nn && drho;
  size_t need = WsCarver::need(use_rho ? p.N * 8 : 0) + WsCarver::need((nn ? n_nn : 0) * 4) +
                2 * WsCarver::need(M * 8) + WsCarver::need(p.N * 8) +
                ztm_pm_adjoint_ws(p, precision, c->num_sms, nn != nullptr) + 4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_rho = wc.take<double>(use_rho ? p.N : 0);
  int* s_nn = wc.take<int>(nn ? n_nn : 0);
  double* s_surf = wc.take<double>(M);
  double* s_w = wc.take<double>(M);
  double* s_g = wc.take<double>(p.N);
  const void *pd = nullptr, *pn = nullptr, *ps, *pw;
  if (use_rho && (rc = ztm_stage_in(c, drho, p.N * 8, dev, s_rho, &pd))) return rc;
  if (nn && (rc = ztm_stage_in(c, nn, n_nn * 4, dev, s_nn, &pn))) return rc;
  if ((rc = ztm_stage_in(c, surf, M * 8, dev, s_surf, &ps))) return rc;
  if ((rc = ztm_stage_in(c, w, M * 8, dev, s_w, &pw))) return rc;
  double* out = dev ? g_drho : s_g;
  rc = ztm_launch_pm_adjoint(c, p, (const double*)pd, (const int*)pn, (const double*)ps,
                             (const double*)pw, out, g->scale, precision, wc);
  if (rc) return rc;
  return ztm_finish(c, dev, g_drho, out, p.N * 8, "point-mass adjoint");
}

extern "C" int ztm_gfm_pointmass_misfit(ztm_ctx* c, const ztm_grid* g, const double* drho,
                                        const int* nn, long long n_nn, const double* surf,
                                        const double* GD, double g0, double gsig, double* ssq,
                                        double* res, double* G, double* g_drho, double* g_g0,
                                        int precision, int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!g || !drho || !surf || !GD || !ssq) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32)
    return ztm_fail(c, ZTM_ERR_ARG, "point-mass precision must be FP64 or FP32");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  if (!(gsig > 0) || !isfinite(g0)) return ztm_fail(c, ZTM_ERR_ARG, "gsig must be > 0, g0 finite");
  PmParams p;
  int rc = ztm_pm_setup(c, g, &p);
  if (rc) return rc;
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  if ((rc = check_nn_host(c, nn, n_nn, p.N, dev))) return rc;
  if (nn) p.nnodes = n_nn;
  const long long M = (long long)g->di * g->dj;
  DevGuard dg(c->device);
  if (!dg.ok) return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  size_t need = WsCarver::need(p.N * 8) + WsCarver::need((nn ? n_nn : 0) * 4) +
                4 * WsCarver::need(M * 8) + WsCarver::need((size_t)std::max(p.ns, 1) * 8) +
                WsCarver::need(p.N * 8) + WsCarver::need(16) + ztm_pm_misfit_ws(p) +
                std::max(ztm_pointmass_ws(p, precision, c->num_sms),
                         g_drho ? ztm_pm_adjoint_ws(p, precision, c->num_sms, nn != nullptr) : 0) +
                4096;
  if ((rc = ztm_ws_reserve(c, need))) return rc;
  WsCarver wc(c->ws);
  double* s_rho = wc.take<double>(p.N);
  int* s_nn = wc.take<int>(nn ? n_nn : 0);
  double* s_surf = wc.take<double>(M);
  double* s_GD = wc.take<double>(M);
  double* s_G = wc.take<double>(M);
  double* s_w = wc.take<double>(M);
  double* s_res = wc.take<double>((size_t)std::max(p.ns, 1));
  double* s_g = wc.take<double>(p.N);
  double* s_out = wc.take<double>(2);
  const void *pd, *pn = nullptr, *ps, *pgd;
  if ((rc = ztm_stage_in(c, drho, p.N * 8, dev, s_rho, &pd))) return rc;
  if (nn && (rc = ztm_stage_in(c, nn, n_nn * 4, dev, s_nn, &pn))) return rc;
  if ((rc = ztm_stage_in(c, surf, M * 8, dev, s_surf, &ps))) return rc;
  if ((rc = ztm_stage_in(c, GD, M * 8, dev, s_GD, &pgd))) return rc;
  double* oG = (dev && G) ? G : s_G;
  double* ores = res ? (dev ? res : s_res) : nullptr;
  double* og = g_drho ? (dev ? g_drho : s_g) : nullptr;
  // the scratch after the fixed slices is shared by the forward and the adjoint
  WsCarver tail = wc;
  rc = ztm_launch_pointmass(c, p, (const double*)pd, (const int*)pn, (const double*)ps, oG,
                            g->scale, precision, tail);
  if (rc) return rc;
  double* oout = s_out;
  WsCarver tail2 = wc;
  rc = ztm_launch_pm_misfit(c, p, oG, (const double*)pgd, g0, gsig, ores, s_w, oout, tail2);
  if (rc) return rc;
  if (og) {
    WsCarver tail3 = tail2;
    rc = ztm_launch_pm_adjoint(c, p, nn ? nullptr : (const double*)pd, (const int*)pn,
                               (const double*)ps, s_w, og, g->scale, precision, tail3);
    if (rc) return rc;
  }
  if (dev) {
    cudaMemcpyAsync(ssq, oout, 8, cudaMemcpyDeviceToDevice, c->stream);
    if (g_g0) cudaMemcpyAsync(g_g0, oout + 1, 8, cudaMemcpyDeviceToDevice, c->stream);
    return ztm_finish(c, true, nullptr, nullptr, 0, "point-mass misfit");
  }
  double h[2] = {0.0, 0.0};
  cudaMemcpyAsync(h, oout, 16, cudaMemcpyDeviceToHost, c->stream);
  if (G) cudaMemcpyAsync(G, oG, M * 8, cudaMemcpyDeviceToHost, c->stream);
  if (res && p.ns > 0) cudaMemcpyAsync(res, ores, (size_t)p.ns * 8, cudaMemcpyDeviceToHost, c->stream);
  if (g_drho) cudaMemcpyAsync(g_drho, og, p.N * 8, cudaMemcpyDeviceToHost, c->stream);
  rc = ztm_finish(c, false, nullptr, nullptr, 0, "point-mass misfit");
  if (rc) return rc;
  *ssq = h[0];
  if (g_g0) *g_g0 = h[1];
  return ZTM_OK;
}
