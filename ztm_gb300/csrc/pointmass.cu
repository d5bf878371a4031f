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
#include <cuda.h>  // CUcontext / CUresult types of the two driver calls below
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <mutex>

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

// Float path by a node list, for grids too deep for the column path below
// (more than 2 * PM_CT levels), in two steps.
//
// 1. Node list (pm_nodes_count / pm_nodes_scan / pm_nodes_write): the
//    selected nodes, in order, in grid units, built once per call (O(nodes),
//    memory bound), stored by pairs: nodes 2p and 2p+1 as the two float4
//    (-i0, -i1, -j0, -j1), (-k0, -k1, w0, w1), so that each packed operand of
//    the gather is one register pair as loaded.  A block covers PM_NB nodes;
//    the blocks' counts are scanned so that each block writes its nodes at
//    its offset in node order; an odd count is padded with a zero mass far
//    away (pm_nodes_pad).
// 2. Gather (pm_gather_f32_kernel): a thread owns a station; the compacted
//    nodes stream through shared memory in tiles of PM_TILE (coalesced float4
//    loads, the next tile's loads in flight while the current one is
//    summed); two nodes per FADD2/FFMA2/FMUL2, the rsqrt on the SFU
//    (rsqrt.approx.ftz).  Plain float sums over 16
//    nodes, Kahan across groups.  grid.y splits the node list; the list's
//    length is read on the device.
constexpr int PM_NB = 1024;  // nodes per block of the node-list kernels
constexpr int PM_NT = 256;   // threads of the node-list kernels (4 nodes each)

__device__ __forceinline__ float pm_rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Node t of the list (t < nnodes): its selection and its float4.  A bad nn
// entry is not selected (and recorded in *err when err is given).
__device__ __forceinline__ bool pm_node(const PmParams& p, const double* __restrict__ drho,
                                        const int* __restrict__ nn, long long t, float4* v,
                                        int* err) {
  const long long n = nn ? (long long)nn[t] : t;
  if (n < 0 || n >= p.N) {
    if (err) atomicOr(err, ZTM_DEVERR_BOUNDS);
    return false;
  }
  const double w = drho[n];
  const bool sel = nn ? true : (fabsf((float)w) > (float)p.thr);
  if (sel) {
    // index map of TFM.cpp:85,97 (fine grid ii = (di-1)*fh+1); N < 2^31
    const int ni = (int)n % p.ii, nj = ((int)n / p.ii) % p.jj, nk = (int)n / (p.ii * p.jj);
    *v = make_float4(-(float)(ni * (1.0 / p.fh)), -(float)(nj * (1.0 / p.fh)),
                     -(float)(nk * (1.0 / p.fv)), (float)w);
  }
  return sel;
}

__global__ void __launch_bounds__(PM_NT)
    pm_nodes_count(PmParams p, const double* __restrict__ drho, const int* __restrict__ nn,
                   int* __restrict__ counts, int* err) {
  __shared__ int s_c;
  if (threadIdx.x == 0) s_c = 0;
  __syncthreads();
  int c = 0;
  for (int q = threadIdx.x; q < PM_NB; q += PM_NT) {
    const long long t = (long long)blockIdx.x * PM_NB + q;
    float4 v;
    if (t < p.nnodes && pm_node(p, drho, nn, t, &v, err)) c++;
  }
  c += __shfl_xor_sync(0xffffffffu, c, 16);
  c += __shfl_xor_sync(0xffffffffu, c, 8);
  c += __shfl_xor_sync(0xffffffffu, c, 4);
  c += __shfl_xor_sync(0xffffffffu, c, 2);
  c += __shfl_xor_sync(0xffffffffu, c, 1);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s_c, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = s_c;
}

// One block: exclusive scan of the nb block counts in place; *total = sum.
__global__ void __launch_bounds__(1024) pm_nodes_scan(int nb, int* __restrict__ counts,
                                                      int* __restrict__ total) {
  __shared__ int s_w[32];
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b0 = 0; b0 < nb; b0 += 1024) {
    const int b = b0 + threadIdx.x;
    const int v = b < nb ? counts[b] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = s_w[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      s_w[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int before = s_carry + (warp ? s_w[warp - 1] : 0) + x - v;
    if (b < nb) counts[b] = before;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s_w[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

__global__ void __launch_bounds__(PM_NT)
    pm_nodes_write(PmParams p, const double* __restrict__ drho, const int* __restrict__ nn,
                   const int* __restrict__ offsets, float4* __restrict__ nodes) {
  __shared__ int s_w[PM_NT / 32];
  __shared__ int s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = offsets[blockIdx.x];
  __syncthreads();
  // PM_NB / PM_NT rounds in node order; each an order-preserving block scan
  for (int q0 = 0; q0 < PM_NB; q0 += PM_NT) {
    const long long t = (long long)blockIdx.x * PM_NB + q0 + threadIdx.x;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    // bad entries were recorded by pm_nodes_count
    const bool sel = t < p.nnodes && pm_node(p, drho, nn, t, &v, nullptr);
    const unsigned bal = __ballot_sync(0xffffffffu, sel);
    const int below = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) s_w[warp] = __popc(bal);
    __syncthreads();
    int wbase = 0;
    for (int w = 0; w < warp; w++) wbase += s_w[w];
    if (sel) {  // pair layout: component c of lane L of pair p at 8p + 2c + L
      const int pos = s_base + wbase + below;
      float* f = reinterpret_cast<float*>(nodes) + 8 * (size_t)(pos >> 1) + (pos & 1);
      f[0] = v.x;
      f[2] = v.y;
      f[4] = v.z;
      f[6] = v.w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < PM_NT / 32; w++) tot += s_w[w];
      s_base += tot;
    }
    __syncthreads();
  }
}

// An odd node count: the second lane of the last pair is a zero mass far away.
__global__ void pm_nodes_pad(const int* __restrict__ total, float4* __restrict__ nodes) {
  const int m = *total;
  if (m & 1) {
    float* f = reinterpret_cast<float*>(nodes) + 8 * (size_t)(m >> 1) + 1;
    f[0] = -1.0e18f;
    f[2] = 0.f;
    f[4] = 0.f;
    f[6] = 0.f;
  }
}

__global__ void __launch_bounds__(PM_TS)
    pm_gather_f32_kernel(PmParams p, const float4* __restrict__ nodes,
                         const int* __restrict__ n_nodes, const double* __restrict__ surf,
                         long long chunk_len, double* __restrict__ partial) {
  __shared__ float4 tile[PM_TILE];
  const int s = blockIdx.x * PM_TS + threadIdx.x;
  const bool active = s < p.ns;
  float i0 = 0.f, j0 = 0.f, k0 = 0.f;
  if (active) {
    const int si = p.bfr + s % p.ni, sj = p.bfr + s / p.ni;
    i0 = (float)si;
    j0 = (float)sj;
    k0 = (float)surf[si + sj * p.di];
  }
  const long long M = *n_nodes;
  const long long n0 = (long long)blockIdx.y * chunk_len;
  const long long n1 = min(M, n0 + chunk_len);
  const float2 I0 = make_float2(i0, i0), J0 = make_float2(j0, j0), K0 = make_float2(k0, k0);
  Kahan acc;
  // this thread's two float4 of the next tile (float4 j holds half of pair
  // j / 2; pairs past the end are zero masses far away)
  auto load = [&](long long j) {
    if (2 * (j >> 1) < n1) return nodes[j];
    return (j & 1) ? make_float4(0.f, 0.f, 0.f, 0.f) : make_float4(-1.0e18f, -1.0e18f, 0.f, 0.f);
  };
  float4 na = load(n0 + threadIdx.x), nb = load(n0 + PM_TS + threadIdx.x);
  for (long long t0 = n0; t0 < n1; t0 += PM_TILE) {
    __syncthreads();  // the previous tile is consumed
    tile[threadIdx.x] = na;
    tile[PM_TS + threadIdx.x] = nb;
    __syncthreads();
    const long long t1 = t0 + PM_TILE;
    na = load(t1 + threadIdx.x);
    nb = load(t1 + PM_TS + threadIdx.x);
    if (!active) continue;
    const int cnt = (int)min((long long)PM_TILE, n1 - t0);
    float2 g = make_float2(0.f, 0.f);
    for (int q = 0; q < cnt; q += 2) {  // an odd count reads the zero-mass pad
      const float4 a = tile[q], b = tile[q + 1];  // nodes q, q + 1 of the tile
      const float2 dx = __fadd2_rn(I0, make_float2(a.x, a.y));
      const float2 dy = __fadd2_rn(J0, make_float2(a.z, a.w));
      const float2 dz = __fadd2_rn(K0, make_float2(b.x, b.y));
      float2 d2 = __fmul2_rn(dz, dz);
      d2 = __ffma2_rn(dy, dy, d2);
      d2 = __ffma2_rn(dx, dx, d2);
      const float2 rs = make_float2(pm_rsqrt_ftz(d2.x), pm_rsqrt_ftz(d2.y));
      const float2 tw = __fmul2_rn(make_float2(b.z, b.w), dz);
      g = __ffma2_rn(__fmul2_rn(tw, __fmul2_rn(rs, rs)), rs, g);
      if ((q & 30) == 30) {  // every 16 nodes
        acc.add(g.x + g.y);
        g = make_float2(0.f, 0.f);
      }
    }
    acc.add(g.x + g.y);
  }
  if (active) partial[(long long)blockIdx.y * p.ns + s] = acc.value();
}

// Float path by node columns (the context entry points).
//
// A run of nodes that shares its horizontal offset needs X^2 + Y^2 once: per
// node pair the gather then forms only Z, r^2, the rsqrt, the weight and the
// product (six packed operations against ten with every node's offsets).  So
// the selected nodes are laid out column by column (fine-grid column
// c = ni + nj*ii, k ascending), each column's run padded to whole pairs:
// 1. pm_cols_count: thread per column, its selected nodes (the threshold, or
//    each node's multiplicity in nn, pm_nn_mark) -> pairs per column;
// 2. pm_nodes_scan over the columns -> each column's first pair and the
//    total;
// 3. pm_cols_write: thread per column, pairs (-k_a, -k_b, w_a, w_b), an odd
//    run closed by a zero mass far away;
// 4. pm_gather_cols_kernel: station tile x column chunk; the pairs of
//    cg_cols columns at a time in shared memory (at most PM_CT pairs), a
//    thread owns a station and forms each column's X^2 + Y^2 once.  Plain
//    float sums over 32 nodes, Kahan across.
constexpr int PM_CT = 512;  // pairs per shared-memory tile of the column gather

// Multiplicity of each node in the nn list (a node listed twice counts
// twice, as in the reference's loop); bad entries are recorded in err.
__global__ void pm_nn_mark(PmParams p, const int* __restrict__ nn, int* __restrict__ mult,
                           int* __restrict__ err) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= p.nnodes) return;
  const long long n = nn[t];
  if (n < 0 || n >= p.N) {
    atomicOr(err, ZTM_DEVERR_BOUNDS);
    return;
  }
  atomicAdd(&mult[n], 1);
}

// Float weight of node n, 0 when it is not selected.
__device__ __forceinline__ float pm_col_weight(const PmParams& p, const double* __restrict__ drho,
                                               const int* __restrict__ mult, long long n) {
  const double w = drho[n];
  if (mult) {
    const int m = mult[n];
    return m ? (float)(w * m) : 0.f;
  }
  return fabsf((float)w) > (float)p.thr ? (float)w : 0.f;
}

// pairs per column, and the column's (-i, -j) in grid units (TFM.cpp:97; in
// double once per column, so that the gather runs no FP64 instruction)
__global__ void pm_cols_count(PmParams p, const double* __restrict__ drho,
                              const int* __restrict__ mult, int* __restrict__ counts,
                              float2* __restrict__ colxy) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  const int ni = (int)(c % p.ii), nj = (int)(c / p.ii);
  colxy[c] = make_float2(-(float)(ni * (1.0 / p.fh)), -(float)(nj * (1.0 / p.fh)));
  int cnt = 0;
  for (int k = 0; k < p.kk; k++)
    if (pm_col_weight(p, drho, mult, c + k * ncols) != 0.f) cnt++;
  counts[c] = (cnt + 1) >> 1;
}

__global__ void pm_cols_write(PmParams p, const double* __restrict__ drho,
                              const int* __restrict__ mult, const int* __restrict__ offs,
                              float4* __restrict__ pairs) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  float4* out = pairs + offs[c];
  int q = 0;
  float ka = 0.f, wa = 0.f;
  for (int k = 0; k < p.kk; k++) {
    const float w = pm_col_weight(p, drho, mult, c + k * ncols);
    if (w == 0.f) continue;
    const float kz = -(float)(k * (1.0 / p.fv));  // -k in grid units (TFM.cpp:97)
    if (q & 1)
      out[q >> 1] = make_float4(ka, kz, wa, w);
    else {
      ka = kz;
      wa = w;
    }
    q++;
  }
  if (q & 1) out[q >> 1] = make_float4(ka, -1.0e18f, wa, 0.f);
}

__global__ void __launch_bounds__(PM_TS)
    pm_gather_cols_kernel(PmParams p, const float4* __restrict__ pairs,
                          const int* __restrict__ offs, const float2* __restrict__ colxy,
                          const double* __restrict__ surf, int cg_cols, int chunk_cols,
                          double* __restrict__ partial) {
  __shared__ float4 tile[PM_CT];
  __shared__ int s_off[PM_CT + 1];
  __shared__ float2 s_xy[PM_CT];
  const int s = blockIdx.x * PM_TS + threadIdx.x;
  const bool active = s < p.ns;
  float i0 = 0.f, j0 = 0.f, k0 = 0.f;
  if (active) {
    const int si = p.bfr + s % p.ni, sj = p.bfr + s / p.ni;
    i0 = (float)si;
    j0 = (float)sj;
    k0 = (float)surf[si + sj * p.di];
  }
  const float2 K0 = make_float2(k0, k0);
  const int ncols = p.ii * p.jj;
  const int c0 = blockIdx.y * chunk_cols, c1 = min(ncols, c0 + chunk_cols);
  Kahan acc;
  for (int cg = c0; cg < c1; cg += cg_cols) {
    const int ce = min(c1, cg + cg_cols);
    __syncthreads();  // the previous group is consumed
    for (int q = threadIdx.x; q <= ce - cg; q += PM_TS) {
      s_off[q] = offs[cg + q];
      if (q < ce - cg) s_xy[q] = colxy[cg + q];
    }
    __syncthreads();
    const int p0 = s_off[0], npair = s_off[ce - cg] - p0;  // <= PM_CT (host)
    for (int q = threadIdx.x; q < npair; q += PM_TS) tile[q] = pairs[p0 + q];
    __syncthreads();
    if (!active) continue;
    for (int c = cg; c < ce; c++) {
      const int a = s_off[c - cg] - p0, b = s_off[c - cg + 1] - p0;
      if (a == b) continue;
      const float2 xy = s_xy[c - cg];
      const float X = i0 + xy.x, Y = j0 + xy.y;
      const float rh = fmaf(X, X, Y * Y);
      const float2 rh2 = make_float2(rh, rh);
      for (int qa = a; qa < b; qa += 16) {
        const int qb = min(b, qa + 16);
        float2 g = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int q = qa; q < qb; q++) {
          const float4 v = tile[q];  // nodes (-k_a, -k_b, w_a, w_b)
          const float2 dz = __fadd2_rn(K0, make_float2(v.x, v.y));
          const float2 d2 = __ffma2_rn(dz, dz, rh2);
          const float2 rs = make_float2(pm_rsqrt_ftz(d2.x), pm_rsqrt_ftz(d2.y));
          const float2 tw = __fmul2_rn(make_float2(v.z, v.w), dz);
          g = __ffma2_rn(__fmul2_rn(tw, __fmul2_rn(rs, rs)), rs, g);
        }
        acc.add(g.x + g.y);
      }
    }
  }
  if (active) partial[(long long)blockIdx.y * p.ns + s] = acc.value();
}

// Double path by node columns: the same layout one node per entry,
// (-k, w) in double, each column's (-i, -j) in double; per node the gather
// forms Z, r^2 = Z^2 + (X^2 + Y^2), the rsqrt and the product in double.
__device__ __forceinline__ double pm_col_weight64(const PmParams& p,
                                                  const double* __restrict__ drho,
                                                  const int* __restrict__ mult, long long n) {
  const double w = drho[n];
  if (mult) {
    const int m = mult[n];
    return m ? w * m : 0.0;
  }
  return fabs(w) > p.thr ? w : 0.0;
}

__global__ void pm_cols_count64(PmParams p, const double* __restrict__ drho,
                                const int* __restrict__ mult, int* __restrict__ counts,
                                double2* __restrict__ colxy) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  const long long ni = c % p.ii, nj = c / p.ii;
  colxy[c] = make_double2(-(ni * (1.0 / p.fh)), -(nj * (1.0 / p.fh)));
  int cnt = 0;
  for (int k = 0; k < p.kk; k++)
    if (pm_col_weight64(p, drho, mult, c + k * ncols) != 0.0) cnt++;
  counts[c] = cnt;
}

__global__ void pm_cols_write64(PmParams p, const double* __restrict__ drho,
                                const int* __restrict__ mult, const int* __restrict__ offs,
                                double2* __restrict__ nodes) {
  const long long ncols = (long long)p.ii * p.jj;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  double2* out = nodes + offs[c];
  int q = 0;
  for (int k = 0; k < p.kk; k++) {
    const double w = pm_col_weight64(p, drho, mult, c + k * ncols);
    if (w != 0.0) out[q++] = make_double2(-(k * (1.0 / p.fv)), w);
  }
}

__global__ void __launch_bounds__(PM_TS)
    pm_gather_cols64_kernel(PmParams p, const double2* __restrict__ nodes,
                            const int* __restrict__ offs, const double2* __restrict__ colxy,
                            const double* __restrict__ surf, int cg_cols, int chunk_cols,
                            double* __restrict__ partial) {
  __shared__ double2 tile[PM_CT];
  __shared__ int s_off[PM_CT + 1];
  __shared__ double2 s_xy[PM_CT];
  const int s = blockIdx.x * PM_TS + threadIdx.x;
  const bool active = s < p.ns;
  double i0 = 0.0, j0 = 0.0, k0 = 0.0;
  if (active) {
    const int si = p.bfr + s % p.ni, sj = p.bfr + s / p.ni;
    i0 = (double)si;
    j0 = (double)sj;
    k0 = surf[si + sj * p.di];
  }
  const int ncols = p.ii * p.jj;
  const int c0 = blockIdx.y * chunk_cols, c1 = min(ncols, c0 + chunk_cols);
  double acc = 0.0;
  for (int cg = c0; cg < c1; cg += cg_cols) {
    const int ce = min(c1, cg + cg_cols);
    __syncthreads();  // the previous group is consumed
    for (int q = threadIdx.x; q <= ce - cg; q += PM_TS) {
      s_off[q] = offs[cg + q];
      if (q < ce - cg) s_xy[q] = colxy[cg + q];
    }
    __syncthreads();
    const int p0 = s_off[0], nnode = s_off[ce - cg] - p0;  // <= PM_CT (host)
    for (int q = threadIdx.x; q < nnode; q += PM_TS) tile[q] = nodes[p0 + q];
    __syncthreads();
    if (!active) continue;
    for (int c = cg; c < ce; c++) {
      const int a = s_off[c - cg] - p0, b = s_off[c - cg + 1] - p0;
      const double2 xy = s_xy[c - cg];
      const double X = i0 + xy.x, Y = j0 + xy.y;
      const double rh = X * X + Y * Y;
#pragma unroll 4
      for (int q = a; q < b; q++) {
        const double2 v = tile[q];  // (-k, w)
        const double dz = k0 + v.x;
        const double rs = rsqrt(dz * dz + rh);
        acc += v.y * dz * (rs * rs * rs);
      }
    }
  }
  if (active) partial[(long long)blockIdx.y * p.ns + s] = acc;
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

// Resident blocks per SM of the gather kernel that a call runs (the float
// path of the context entry points is the column kernel, or the compacted
// list for very deep grids).
int pm_occupancy(int precision, bool compacted, bool cols = false) {
  int occ = 0;
  cudaError_t e;
  if (precision == ZTM_PREC_FP64 && cols)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pm_gather_cols64_kernel, PM_TS, 0);
  else if (precision == ZTM_PREC_FP64)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pm_gather_kernel<true>, PM_TS, 0);
  else if (cols)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pm_gather_cols_kernel, PM_TS, 0);
  else if (compacted)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pm_gather_f32_kernel, PM_TS, 0);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pm_gather_kernel<false>, PM_TS, 0);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    occ = 1;
  }
  return occ;
}

// Station tiles x node chunks: about four waves of resident blocks (occ per
// SM), chunks of at least 1024 nodes.
void pm_shape(const PmParams& p, int num_sms, int occ, int* tiles, int* chunks, long long* clen) {
  *tiles = (p.ns + PM_TS - 1) / PM_TS;
  if (*tiles < 1) *tiles = 1;
  long long want =
      std::max(1LL, (4LL * occ * std::max(num_sms, 1) + *tiles - 1) / *tiles);
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

// Entries of one column's run: node pairs (float) or nodes (double).
int pm_col_entries(const PmParams& p, bool f64) { return f64 ? p.kk : (p.kk + 1) / 2; }
// The column path: a column's run fits one shared-memory tile.
bool pm_use_cols(const PmParams& p, bool f64 = false) { return pm_col_entries(p, f64) <= PM_CT; }

// Column gather shape: station tiles x column chunks of whole column groups
// (cg_cols columns, at most PM_CT pairs), about sixteen waves of resident
// blocks (62.4 ms at four waves, 61.2 at eight, 60.7 at sixteen on the
// 256x256x65-node grid).
void pm_cols_shape(const PmParams& p, int num_sms, bool f64, int* tiles, int* chunks,
                   int* chunk_cols, int* cg_cols) {
  const int occ = pm_occupancy(f64 ? ZTM_PREC_FP64 : ZTM_PREC_FP32, true, true);
  *tiles = std::max(1, (p.ns + PM_TS - 1) / PM_TS);
  const long long ncols = (long long)p.ii * p.jj;
  *cg_cols = std::max(1, PM_CT / std::max(1, pm_col_entries(p, f64)));
  const long long want = std::max(1LL, (16LL * occ * std::max(num_sms, 1) + *tiles - 1) / *tiles);
  const long long groups = (ncols + *cg_cols - 1) / *cg_cols;
  const long long ch = std::max(1LL, std::min(std::min(want, groups), 65535LL));
  const long long per = (groups + ch - 1) / ch;  // groups per chunk
  *chunk_cols = (int)(per * *cg_cols);
  *chunks = (int)((ncols + *chunk_cols - 1) / *chunk_cols);
}

}  // namespace

void ztm_scan_ints(cudaStream_t s, int n, int* counts, int* total) {
  pm_nodes_scan<<<1, 1024, 0, s>>>(n, counts, total);
}

size_t ztm_pointmass_ws(const PmParams& p, int precision, int num_sms) {
  const bool f64 = precision == ZTM_PREC_FP64;
  if (pm_use_cols(p, f64)) {  // the node columns
    int ct, cc, ccols, cg;
    pm_cols_shape(p, num_sms, f64, &ct, &cc, &ccols, &cg);
    const long long ncols = (long long)p.ii * p.jj;
    const size_t entries = f64 ? (size_t)p.N + 2 : (size_t)((p.N + ncols) / 2 + 2);
    return WsCarver::need((size_t)cc * std::max(p.ns, 1) * sizeof(double)) +
           WsCarver::need((size_t)(ncols + 1) * sizeof(int)) +
           WsCarver::need((size_t)ncols * 16) + WsCarver::need(entries * 16) +
           WsCarver::need((size_t)p.N * sizeof(int));  // nn multiplicities
  }
  int tiles, chunks;
  long long len;
  pm_shape(p, num_sms, pm_occupancy(precision, true), &tiles, &chunks, &len);
  size_t w = WsCarver::need((size_t)chunks * std::max(p.ns, 1) * sizeof(double));
  if (precision != ZTM_PREC_FP64) {  // the float node list
    const long long nb = std::max(1LL, (p.nnodes + PM_NB - 1) / PM_NB);
    w += WsCarver::need((size_t)(std::max(p.nnodes, 1LL) + 2) * sizeof(float4)) +
         WsCarver::need((size_t)nb * sizeof(int)) + WsCarver::need(sizeof(int));
  }
  return w;
}

int ztm_launch_pointmass(ztm_ctx* c, const PmParams& p, const double* d_drho,
                         const int* d_nn, const double* d_surf, double* d_G,
                         double scale, int precision, WsCarver& wc) {
  const bool f64 = precision == ZTM_PREC_FP64;
  const bool cols = pm_use_cols(p, f64);
  int tiles, chunks, chunk_cols = 0, cg_cols = 0;
  long long len = 0;
  if (cols)
    pm_cols_shape(p, c->num_sms, f64, &tiles, &chunks, &chunk_cols, &cg_cols);
  else
    pm_shape(p, c->num_sms, pm_occupancy(precision, true), &tiles, &chunks, &len);
  double* partial = wc.take<double>((size_t)chunks * std::max(p.ns, 1));
  if (p.ns > 0 && p.nnodes > 0) {
    dim3 grid(tiles, chunks);
    if (cols && f64) {
      const long long ncols = (long long)p.ii * p.jj;
      int* offs = wc.take<int>((size_t)ncols + 1);
      double2* colxy = wc.take<double2>((size_t)ncols);
      double2* nodes = wc.take<double2>((size_t)p.N + 2);
      int* mult = nullptr;
      if (d_nn) {  // the listed nodes, with their multiplicities
        mult = wc.take<int>((size_t)p.N);
        cudaMemsetAsync(mult, 0, (size_t)p.N * sizeof(int), c->stream);
        pm_nn_mark<<<(unsigned)((p.nnodes + 255) / 256), 256, 0, c->stream>>>(p, d_nn, mult,
                                                                             c->d_err);
        c->launches++;
      }
      const unsigned cb = (unsigned)((ncols + 255) / 256);
      pm_cols_count64<<<cb, 256, 0, c->stream>>>(p, d_drho, mult, offs, colxy);
      pm_nodes_scan<<<1, 1024, 0, c->stream>>>((int)ncols, offs, offs + ncols);
      pm_cols_write64<<<cb, 256, 0, c->stream>>>(p, d_drho, mult, offs, nodes);
      {
        ZtmProf prof_(c, "pointmass");
        pm_gather_cols64_kernel<<<grid, PM_TS, 0, c->stream>>>(p, nodes, offs, colxy, d_surf,
                                                              cg_cols, chunk_cols, partial);
      }
      c->launches += 4;
    } else if (precision == ZTM_PREC_FP64) {
      ZtmProf prof_(c, "pointmass");
      pm_gather_kernel<true><<<grid, PM_TS, 0, c->stream>>>(p, d_drho, d_nn, d_surf, len, partial,
                                                            c->d_err);
      c->launches++;
    } else if (cols) {
      const long long ncols = (long long)p.ii * p.jj;
      int* offs = wc.take<int>((size_t)ncols + 1);
      float2* colxy = wc.take<float2>((size_t)ncols);
      float4* pairs = wc.take<float4>((size_t)((p.N + ncols) / 2 + 2));
      int* mult = nullptr;
      if (d_nn) {  // the listed nodes, with their multiplicities
        mult = wc.take<int>((size_t)p.N);
        cudaMemsetAsync(mult, 0, (size_t)p.N * sizeof(int), c->stream);
        pm_nn_mark<<<(unsigned)((p.nnodes + 255) / 256), 256, 0, c->stream>>>(p, d_nn, mult,
                                                                             c->d_err);
        c->launches++;
      }
      const unsigned cb = (unsigned)((ncols + 255) / 256);
      pm_cols_count<<<cb, 256, 0, c->stream>>>(p, d_drho, mult, offs, colxy);
      pm_nodes_scan<<<1, 1024, 0, c->stream>>>((int)ncols, offs, offs + ncols);
      pm_cols_write<<<cb, 256, 0, c->stream>>>(p, d_drho, mult, offs, pairs);
      {
        ZtmProf prof_(c, "pointmass");
        pm_gather_cols_kernel<<<grid, PM_TS, 0, c->stream>>>(p, pairs, offs, colxy, d_surf,
                                                            cg_cols, chunk_cols, partial);
      }
      c->launches += 4;
    } else {
      const long long nb = (p.nnodes + PM_NB - 1) / PM_NB;
      if (nb > (1LL << 31) - 1) return ztm_fail(c, ZTM_ERR_RANGE, "too many point-mass nodes");
      float4* nodes = wc.take<float4>((size_t)p.nnodes + 2);  // + the pad of an odd count
      int* counts = wc.take<int>((size_t)nb);
      int* total = wc.take<int>(1);
      pm_nodes_count<<<(unsigned)nb, PM_NT, 0, c->stream>>>(p, d_drho, d_nn, counts, c->d_err);
      pm_nodes_scan<<<1, 1024, 0, c->stream>>>((int)nb, counts, total);
      pm_nodes_write<<<(unsigned)nb, PM_NT, 0, c->stream>>>(p, d_drho, d_nn, counts, nodes);
      pm_nodes_pad<<<1, 1, 0, c->stream>>>(total, nodes);
      {
        ZtmProf prof_(c, "pointmass");
        pm_gather_f32_kernel<<<grid, PM_TS, 0, c->stream>>>(p, nodes, total, d_surf, len, partial);
      }
      c->launches += 5;
    }
  } else {
    chunks = 0;
  }
  double factor = scale * 66.7 / ((double)p.fh * p.fh * p.fv);
  int M = p.di * p.dj;
  pm_finalize_kernel<<<(M + 255) / 256, 256, 0, c->stream>>>(p, chunks, partial, factor, d_G);
  c->launches++;
  return ztm_after_launch(c, "point-mass kernels");
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the point-mass forward.
//
// Some callers cannot allocate device memory when they need a forward: a host
// application that hands the GPU to this code with a fixed memory budget set
// up front (and treats any later cudaMalloc as a failure), code that runs
// while a stream is being captured into a CUDA graph (cudaMalloc is not
// allowed there), or a real-time inversion loop that must not pay for, or
// risk, an allocation inside its iterations.  For them
// ztm_gfm_pointmass_noalloc computes the same sum as ztm_gfm_pointmass with
// the full-grid gather pm_gather_kernel (nodes in grid order, the threshold
// applied on the fly; not the node-column gather of the context entry points,
// which needs a workspace for its column layout, so its rates are those of
// pm_gather_kernel) and keeps all of its scratch (the per-chunk partial sums
// and the error word) in the fixed array below.  It needs no context, does no
// host<->device staging, and calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// Limits and sharing:
//   * ZTM_NOALLOC_SCRATCH_BYTES (4 MiB) per GPU, reserved in every GPU that
//     loads the library for as long as the library stays loaded;
//   * at most (4 MiB - 256) / 8 = 524,256 interior stations (fewer node
//     chunks are used when the stations fill the array);
//   * every call on a device writes the same array: calls that may overlap
//     on that GPU (different streams, or threads without ordering) race and
//     give wrong results; serialise them on one stream;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, which may load the module onto the device); make
//     that first call before any stream capture begins.  The address is kept
//     per device and CUDA context: after a cudaDeviceReset the next call looks
//     it up again (that call is then a first call).
#define ZTM_NOALLOC_SCRATCH_BYTES (4u << 20)
static __device__ __align__(256) unsigned char g_pm_scratch[ZTM_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
struct NoallocSlot {
  unsigned long long ctx_id = 0;  // the CUDA context the address belongs to
  void* addr = nullptr;
};
NoallocSlot g_noalloc[NOALLOC_MAX_DEVICES];

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current CUDA context, 0 when there is
// none yet (or the driver cannot say).  The driver functions are reached
// through the runtime, so the library does not link libcuda itself.
unsigned long long current_ctx_id() {
  static PfnCtxGetCurrent get_cur = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    void *f1 = nullptr, *f2 = nullptr;
    const cudaError_t e1 =
        cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    const cudaError_t e2 =
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e1 == cudaSuccess && e2 == cudaSuccess && q1 == cudaDriverEntryPointSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      get_cur = reinterpret_cast<PfnCtxGetCurrent>(f1);
      get_id = reinterpret_cast<PfnCtxGetId>(f2);
    }
  });
  if (!get_cur || !get_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}
}  // namespace

extern "C" int ztm_gfm_pointmass_noalloc(const ztm_grid* g, const double* drho,
                                         const double* surf, double* G, int precision,
                                         void* stream) {
  if (!g || !drho || !surf || !G) return ZTM_ERR_ARG;
  if (precision != ZTM_PREC_FP64 && precision != ZTM_PREC_FP32) return ZTM_ERR_ARG;
  // an error left pending by the caller's earlier work is not this call's:
  // report it without clearing it, so that its owner still sees it
  if (cudaPeekAtLastError() != cudaSuccess) return ZTM_ERR_CUDA;
  if (g->di < 1 || g->dj < 1 || g->dk < 1 || g->fh < 1 || g->fv < 1 || g->bfr < 0 ||
      !(g->threshold >= 0) || !isfinite(g->scale))
    return ZTM_ERR_ARG;
  int dev = -1, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    return ZTM_ERR_NODEV;
  }
  if (dev >= NOALLOC_MAX_DEVICES) return ZTM_ERR_RANGE;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return ZTM_ERR_CUDA;
  }
  PmParams p;
  p.di = g->di; p.dj = g->dj; p.fh = g->fh; p.fv = g->fv; p.bfr = g->bfr;
  p.ii = (g->di - 1) * g->fh + 1;
  p.jj = (g->dj - 1) * g->fh + 1;
  p.kk = (g->dk - 1) * g->fv + 1;
  const long long N = (long long)p.ii * p.jj * p.kk;
  if (N > (1LL << 31) - 1) return ZTM_ERR_RANGE;
  p.ni = std::max(0, g->di - 2 * g->bfr);
  p.nj = std::max(0, g->dj - 2 * g->bfr);
  p.ns = p.ni * p.nj;
  p.thr = g->threshold;
  p.nnodes = N;
  p.N = N;
  const long long cap = (ZTM_NOALLOC_SCRATCH_BYTES - 256) / sizeof(double);
  if (p.ns > cap) return ZTM_ERR_RANGE;  // more interior stations than the array holds

  // set-up once per device and context: the host-side name of the array is
  // not a device address; ask the runtime for the address on this device
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSlot& slot = g_noalloc[dev];
    const unsigned long long id = current_ctx_id();
    if (!slot.addr || id == 0 || id != slot.ctx_id) {
      void* a = nullptr;
      if (cudaGetSymbolAddress(&a, g_pm_scratch) != cudaSuccess || !a) {
        cudaGetLastError();  // raised here (none was pending at entry)
        return ZTM_ERR_CUDA;
      }
      slot.addr = a;
      slot.ctx_id = current_ctx_id();  // the lookup made the context current
    }
    base = slot.addr;
  }
  int* err = reinterpret_cast<int*>(base);
  double* partial = reinterpret_cast<double*>(static_cast<char*>(base) + 256);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  int tiles, chunks;
  long long len;
  pm_shape(p, nsm, pm_occupancy(precision, false), &tiles, &chunks, &len);
  if (p.ns > 0 && (long long)chunks * p.ns > cap) {  // fewer, longer node chunks
    chunks = (int)std::max(1LL, cap / p.ns);
    len = (p.nnodes + chunks - 1) / chunks;
    len = ((len + PM_TILE - 1) / PM_TILE) * PM_TILE;
    chunks = (int)((p.nnodes + len - 1) / len);
  }
  // every (chunk, station) partial is rewritten below; only the error word
  // has to start at zero
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) {
    cudaGetLastError();
    return ZTM_ERR_CUDA;
  }
  if (p.ns > 0 && p.nnodes > 0) {
    dim3 grid(tiles, chunks);
    if (precision == ZTM_PREC_FP64)
      pm_gather_kernel<true><<<grid, PM_TS, 0, s>>>(p, drho, nullptr, surf, len, partial, err);
    else
      pm_gather_kernel<false><<<grid, PM_TS, 0, s>>>(p, drho, nullptr, surf, len, partial, err);
  } else {
    chunks = 0;
  }
  const double factor = g->scale * 66.7 / ((double)p.fh * p.fh * p.fv);
  const int M = p.di * p.dj;
  pm_finalize_kernel<<<(M + 255) / 256, 256, 0, s>>>(p, chunks, partial, factor, G);
  // a launch error here is this call's own (none was pending at entry)
  if (cudaGetLastError() != cudaSuccess) return ZTM_ERR_CUDA;
  return ZTM_OK;
}
