// pointmass.cu - the reference's point-mass gravity model on sm_103a.
//
// Model (TFM.cpp:96-98, GFM_GPU.cu:17-22): every selected fine-grid node n at
// (i,j,k) = ((n%ii)/fh, ((n/ii)%jj)/fh, (n/(ii*jj))/fv) is a point mass, and
// an interior station (i0, j0, k0=surf[i0+j0*di]) receives
//     66.7/(fh^2 fv) * drho[n] * (k0-k) / ((i0-i)^2+(j0-j)^2+(k0-k)^2)^1.5 .
//
// The reference GF kernel scatters: one thread per node, one float atomicAdd
// per (node, station) pair into the same station address across a warp.
// Here the sum is a gather: a thread owns a station, nodes stream through
// shared memory tile by tile (one broadcast read per pair), the per-thread
// sum stays in registers, and a split over node chunks writes per-chunk
// partials that a second kernel adds in a fixed order.  No atomics, so the
// result is bitwise reproducible.
#include <cuda_runtime.h>

#include <algorithm>

#include "ztm_internal.cuh"

namespace {

constexpr int PM_TS = 128;    // stations (threads) per block
constexpr int PM_TILE = 256;  // nodes per shared-memory tile

struct __align__(16) Node64 {
  double x, y, z, w;
};

template <bool F64>
struct NodeT;
template <>
struct NodeT<true> {
  using T = double;
  using V = Node64;
};
template <>
struct NodeT<false> {
  using T = float;
  using V = float4;
};

// grid.x: station tiles, grid.y: node chunks.  partial[chunk*ns + s].
template <bool F64>
__global__ void __launch_bounds__(PM_TS)
    pm_gather_kernel(PmParams p, const double* __restrict__ drho,
                     const int* __restrict__ nn, const double* __restrict__ surf,
                     long long chunk_len, double* __restrict__ partial, int* err) {
  using T = typename NodeT<F64>::T;
  using V = typename NodeT<F64>::V;
  __shared__ V tile[PM_TILE];

  const int s = blockIdx.x * PM_TS + threadIdx.x;
  const bool active = s < p.ns;
  T i0 = 0, j0 = 0, k0 = 0;
  if (active) {
    int si = p.bfr + s % p.ni, sj = p.bfr + s / p.ni;
    i0 = (T)si;
    j0 = (T)sj;
    double kd = surf[si + sj * p.di];
    k0 = (T)kd;  // float mode: the station height travels as float, as S.dat does
  }
  const long long n0 = (long long)blockIdx.y * chunk_len;
  const long long n1 = min(p.nnodes, n0 + chunk_len);
  const double ifh = 1.0 / p.fh, ifv = 1.0 / p.fv;
  const long long plane = (long long)p.ii * p.jj;

  double acc64 = 0.0;
  Kahan acc32;
  for (long long t0 = n0; t0 < n1; t0 += PM_TILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < PM_TILE; q += PM_TS) {
      long long t = t0 + q;
      V v;
      v.x = v.y = v.z = v.w = (T)0;
      if (t < n1) {
        long long n = nn ? (long long)nn[t] : t;
        if (n < 0 || n >= p.N) {  // bad list entry: record it, contribute nothing
          atomicOr(err, ZTM_DEVERR_BOUNDS);
          tile[q] = v;
          continue;
        }
        double w = drho[n];
        bool sel = nn ? true : (fabs(w) > p.thr);
        if (!F64) sel = nn ? true : (fabsf((float)w) > (float)p.thr);
        // index map of TFM.cpp:85,97 (fine grid ii = (di-1)*fh+1)
        long long ni = n % p.ii, nj = (n / p.ii) % p.jj, nk = n / plane;
        v.x = (T)(ni * ifh);
        v.y = (T)(nj * ifh);
        v.z = (T)(nk * ifv);
        v.w = sel ? (T)w : (T)0;
      }
      tile[q] = v;
    }
    __syncthreads();
    const int cnt = (int)min((long long)PM_TILE, n1 - t0);
    if (active) {
#pragma unroll 4
      for (int q = 0; q < cnt; q++) {
        V v = tile[q];
        if (v.w != (T)0) {  // uniform across the warp: every lane reads node q
          T dx = i0 - v.x, dy = j0 - v.y, dz = k0 - v.z;
          T d2 = dx * dx + dy * dy + dz * dz;
          if (F64) {
            double rs = rsqrt((double)d2);
            acc64 += (double)v.w * (double)dz * (rs * rs * rs);
          } else {
            float rs = rsqrtf((float)d2);
            acc32.add((float)v.w * (float)dz * (rs * rs * rs));
          }
        }
      }
    }
  }
  if (active) partial[(long long)blockIdx.y * p.ns + s] = F64 ? acc64 : acc32.value();
}

// G[m] = factor * sum_chunks partial for interior m, 0 elsewhere.
__global__ void pm_finalize_kernel(PmParams p, int nchunks,
                                   const double* __restrict__ partial,
                                   double factor, double* __restrict__ G) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= p.di * p.dj) return;
  int i0 = m % p.di, j0 = m / p.di;
  double g = 0.0;
  if (i0 >= p.bfr && i0 < p.di - p.bfr && j0 >= p.bfr && j0 < p.dj - p.bfr) {
    int s = (i0 - p.bfr) + (j0 - p.bfr) * p.ni;
    for (int c = 0; c < nchunks; c++) g += partial[(long long)c * p.ns + s];
    g *= factor;
  }
  G[m] = g;
}

void pm_shape(const PmParams& p, int num_sms, int* tiles, int* chunks, long long* clen) {
  *tiles = (p.ns + PM_TS - 1) / PM_TS;
  if (*tiles < 1) *tiles = 1;
  long long want = std::max(1LL, (long long)(8 * std::max(num_sms, 1)) / *tiles);
  long long maxc = std::max(1LL, (p.nnodes + 1023) / 1024);
  long long ch = std::min(want, maxc);
  ch = std::min(ch, 65535LL);
  long long len = (p.nnodes + ch - 1) / ch;
  len = ((len + PM_TILE - 1) / PM_TILE) * PM_TILE;
  if (len < PM_TILE) len = PM_TILE;
  ch = (p.nnodes + len - 1) / len;
  if (ch < 1) ch = 1;
  *chunks = (int)ch;
  *clen = len;
}

}  // namespace

size_t ztm_pointmass_ws(const PmParams& p, int precision, int num_sms) {
  (void)precision;
  int tiles, chunks;
  long long len;
  pm_shape(p, num_sms, &tiles, &chunks, &len);
  return WsCarver::need((size_t)chunks * std::max(p.ns, 1) * sizeof(double));
}

int ztm_launch_pointmass(ztm_ctx* c, const PmParams& p, const double* d_drho,
                         const int* d_nn, const double* d_surf, double* d_G,
                         double scale, int precision, WsCarver& wc) {
  int tiles, chunks;
  long long len;
  pm_shape(p, c->num_sms, &tiles, &chunks, &len);
  double* partial = wc.take<double>((size_t)chunks * std::max(p.ns, 1));
  if (p.ns > 0 && p.nnodes > 0) {
    dim3 grid(tiles, chunks);
    if (precision == ZTM_PREC_FP64)
      {
        ZtmProf prof_(c, "pointmass");
        pm_gather_kernel<true><<<grid, PM_TS, 0, c->stream>>>(p, d_drho, d_nn, d_surf, len, partial, c->d_err);
      }
    else
      {
        ZtmProf prof_(c, "pointmass");
        pm_gather_kernel<false><<<grid, PM_TS, 0, c->stream>>>(p, d_drho, d_nn, d_surf, len, partial, c->d_err);
      }
    c->launches++;
  } else {
    chunks = 0;
  }
  double factor = scale * 66.7 / ((double)p.fh * p.fh * p.fv);
  int M = p.di * p.dj;
  pm_finalize_kernel<<<(M + 255) / 256, 256, 0, c->stream>>>(p, chunks, partial, factor, d_G);
  c->launches++;
  return ztm_after_launch(c, "point-mass kernels");
}
