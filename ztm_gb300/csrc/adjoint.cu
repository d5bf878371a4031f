// adjoint.cu - transposed sum of the prism forward (dmisfit/drho).
//
// For misfit 0.5*|gz - d|^2 and residual r = gz - d, the density gradient is
//   g_rho[p] = sum_s r[s] * dgz[s]/drho[p] = G*1e5 * sum_s r[s] * U(s, p),
// the transpose of the forward sum (prism.cu) with the same pair function.
// The reference has no adjoint: its optimiser differentiates every gravity
// parameter by a full forward run (TFM.cpp:124-135); this is what replaces
// those gravity columns.
//
//   FP64 plain  thread per mesh vertex (the station-weighted corner function
//               Psi(v), vertex sharing), stations streamed through shared memory,
//               8-corner closed form in double; station chunks reduced in a
//               fixed order.
//   MIXED/FP32  far pairs: thread per (column, group of 32 layers) and
//               station slice, the column's horizontal offsets and polynomial
//               computed once per station and the far-field expansion per
//               layer in float (second order where the whole warp is far
//               enough), float sums over 32 stations, compensated beyond; the
//               slices meet in g_rho by double atomics.  Near pairs (prisms in
//               the station's near region): one warp per station computes
//               Phi once per vertex into its block's slice of a global
//               scratch, combines the 8 corners of each near prism and adds
//               r[s]*U to g_rho with double atomics.  Both are items of one
//               persistent grid's work queue, the near items spread evenly
//               among the far items, so that the near regions' FP64 work
//               runs beside the far fields' FP32 work on every SM.  g_rho is
//               zeroed first; the atomics make the last bits order-dependent.
#include <cuda_runtime.h>

#include <algorithm>

#include "prism_common.cuh"
#include "ztm_internal.cuh"

namespace {

constexpr int ADJ_TS = 128;
constexpr int ADJ_LG = 32;     // layers per thread in the far kernel
constexpr int ADJ_STILE = 64;  // stations per shared-memory tile
constexpr int ADJ_SGRP = 32;   // stations per float sum

constexpr int ADJ_NEAR_ST = 8;  // stations per near item (two per warp)

struct AdjArgs {
  MeshConst k;
  MeshDesc m;
  int ns;
  const float4* sf;
  const int4* si;
  const short2* iv;   // near-region intervals [station][box column]
  const int2* lr;     // per-station near layer range
  const double* sxyz;
  const double* res;
  double scale;       // G5 * L0 * Vn: far sums to gradient units
  double G5;
  int slice;          // stations per far item (a multiple of ADJ_STILE)
  int tiles, slices;  // far items: column tiles x station slices
  int n_near;         // near items (ADJ_NEAR_ST stations each)
  int cap;            // near-box vertices per warp's scratch
  double* phi;        // [grid][warps][cap] near-box vertex values
  int* counter;       // next work item (zeroed before the launch)
  double* g;
};

// Shared memory of a far item: a tile of stations and the double sums of
// each thread's layers.
struct AdjSmem {
  float4 f[ADJ_STILE];
  int4 b[ADJ_STILE];   // the station's near box columns x0, x1, y0, y1
  float4 h[ADJ_STILE]; // the home cell indices as floats (exact)
  float r[ADJ_STILE];
  float4 z[ADJ_STILE][ADJ_LG / 4];  // the station's Z at the item's 32 layers
  float2 acc[ADJ_LG][ADJ_TS];  // compensated float sums (sum, compensation)
};

// Compensated float add of x into k = (sum, compensation).
__device__ __forceinline__ void kahan2(float2& k, float x) {
  const float y = x - k.y;
  const float t = k.x + y;
  k.y = (t - k.x) - y;
  k.x = t;
}

// Far item (column tile bx, station slice by): thread per (column, group of
// 32 layers), g[p] += G5*L0*Vn * sum.  A thread sums its column's 32 layers
// over the slice's stations: float over 32 stations (packed, two layers per
// lane pair), then compensated float sums in shared memory (no FP64
// instruction per group: GB300's FP64 pipe is slow), then one double atomic per
// layer into g.  The per-(station, column) setup (offsets, the horizontal
// polynomial, the near box test) is shared by the 32 layers.
__device__ __forceinline__ void adj_far_item(const AdjArgs& a, int bx, int by, AdjSmem& sm) {
  const MeshConst& k = a.k;
  // column tiles of one layer group each: a block's threads share the
  // group, so a station's Z values are formed once per block (shared memory)
  const int tpg = (k.ncols + ADJ_TS - 1) / ADJ_TS;  // column tiles per layer group
  const int lg = bx / tpg;
  const int cc = (bx % tpg) * ADJ_TS + threadIdx.x;
  const bool active = cc < k.ncols;
  const int c = active ? cc : 0;
  const int ix = c % k.nx, iy = c / k.nx;
  const int l0 = lg * ADJ_LG;
  const float fix = (float)ix, fiy = (float)iy, fl0 = (float)l0;
  const FarCoef fc = k.fc;
#pragma unroll
  for (int j = 0; j < ADJ_LG; j++) sm.acc[j][threadIdx.x] = make_float2(0.f, 0.f);
  // this item's slice of the stations
  const int sb = by * a.slice, se = min(a.ns, sb + a.slice);
  for (int s0 = sb; s0 < se; s0 += ADJ_STILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < ADJ_STILE; q += ADJ_TS) {
      const int s = s0 + q;
      if (s < se) {
        const int4 i = a.si[s];
        const NearBox b = near_box(i, k);
        sm.f[q] = a.sf[s];
        sm.b[q] = make_int4(b.x0, b.x1, b.y0, b.y1);
        sm.h[q] = make_float4((float)i.x, (float)i.y, (float)i.z, 0.f);
        sm.r[q] = (float)a.res[s];
        const float zg = fmaf(fl0 - (float)i.z, k.dzn, a.sf[s].z);
#pragma unroll
        for (int j = 0; j < ADJ_LG / 4; j++)
          sm.z[q][j] = make_float4(fmaf((float)(4 * j), k.dzn, zg), fmaf((float)(4 * j + 1), k.dzn, zg),
                                   fmaf((float)(4 * j + 2), k.dzn, zg), fmaf((float)(4 * j + 3), k.dzn, zg));
      } else {
        sm.f[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        sm.b[q] = make_int4(1, 0, 1, 0);
        sm.h[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        sm.r[q] = 0.f;
#pragma unroll
        for (int j = 0; j < ADJ_LG / 4; j++) sm.z[q][j] = make_float4(1.f, 1.f, 1.f, 1.f);
      }
    }
    __syncthreads();
    if (!active) continue;
    const int cnt = min(ADJ_STILE, se - s0);
    for (int q0 = 0; q0 < cnt; q0 += ADJ_SGRP) {
      float2 gs[ADJ_LG / 2];
#pragma unroll
      for (int j = 0; j < ADJ_LG / 2; j++) gs[j] = make_float2(0.f, 0.f);
      const int q1 = min(cnt, q0 + ADJ_SGRP);
      for (int q = q0; q < q1; q++) {
        const float4 f = sm.f[q];
        const float4 hf = sm.h[q];
        const float X = fmaf(hf.x - fix, k.dxn, f.x);
        const float Y = fmaf(hf.y - fiy, k.dyn, f.y);
        const float X2 = X * X, Y2 = Y * Y, rh = X2 + Y2;
        const int4 b = sm.b[q];
        bool ncl = ix >= b.x && ix <= b.y && iy >= b.z && iy <= b.w;
        int elo = k.nz;
        unsigned espan = 0u;
        if (ncl) {  // the column's near-region layers for this station
          const short2 tv =
              a.iv[(size_t)(s0 + q) * k.nslots + (ix - b.x) + (b.y - b.x + 1) * (iy - b.z)];
          if (tv.x <= tv.y) {
            elo = tv.x;
            espan = (unsigned)(tv.y - tv.x);
          } else {
            ncl = false;
          }
        }
        // Z of layers l0 + 2j, l0 + 2j + 1
        auto zof = [&](int j) {
          const float4 z4 = sm.z[q][j >> 1];
          return (j & 1) ? make_float2(z4.z, z4.w) : make_float2(z4.x, z4.y);
        };
        const float2 w2 = make_float2(sm.r[q], sm.r[q]);
        float2 v[ADJ_LG / 2];
        // the warp's columns all far enough for the second-order form (the
        // lanes of a warp share the station, so this is mostly uniform),
        // which needs only C2t = a0 - a1 rh of the column polynomial
        if (__all_sync(__activemask(), rh >= k.rh_t2)) {
          const float c2 = fmaf(-fc.a1, rh, fmaf(X2, fc.cA, Y2 * fc.cB));
          const float2 c2t = make_float2(c2, c2);
          ColPoly2 cp2;
          cp2.rh = make_float2(rh, rh);
          cp2.a1 = make_float2(fc.a1, fc.a1);
          cp2.C2 = cp2.C3 = cp2.C4 = cp2.C5 = cp2.C6 = make_float2(0.f, 0.f);  // unused by the form
#pragma unroll
          for (int j = 0; j < ADJ_LG / 2; j++) v[j] = far_unit2_t2(zof(j), cp2, c2t);
        } else {
          const ColPoly2 cp2 = col_poly2(col_poly(X, Y, fc), fc.a1);
#pragma unroll
          for (int j = 0; j < ADJ_LG / 2; j++) v[j] = far_unit2(zof(j), cp2);
        }
        if (ncl || l0 + ADJ_LG > k.nz) {
#pragma unroll
          for (int j = 0; j < ADJ_LG / 2; j++) {
            const int la = l0 + 2 * j, lb = la + 1;
            if (((unsigned)(la - elo) <= espan) || la >= k.nz) v[j].x = 0.f;
            if (((unsigned)(lb - elo) <= espan) || lb >= k.nz) v[j].y = 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < ADJ_LG / 2; j++) gs[j] = __ffma2_rn(w2, v[j], gs[j]);
      }
      // the group's float sums into the compensated accumulators
#pragma unroll
      for (int j = 0; j < ADJ_LG / 2; j++) {
        kahan2(sm.acc[2 * j][threadIdx.x], gs[j].x);
        kahan2(sm.acc[2 * j + 1][threadIdx.x], gs[j].y);
      }
    }
  }
  if (!active) return;
  const long long plane = (long long)k.ncols;
#pragma unroll
  for (int j = 0; j < ADJ_LG; j++) {
    const int l = l0 + j;
    if (l < k.nz) {
      const float2 kc = sm.acc[j][threadIdx.x];
      atomicAdd(&a.g[c + plane * l], a.scale * ((double)kc.x - (double)kc.y));
    }
  }
}

// Near region of station s, by one warp: Phi at every vertex of the near
// box's layer range into the warp's scratch (phi, cap values), then per near
// prism the signed 8-corner sum, scaled by r[s], added to g with double
// atomics.
template <typename T>
__device__ __forceinline__ void adj_near_station(const AdjArgs& a, int s, T* phi, int lane) {
  const MeshConst& k = a.k;
  const MeshDesc& m = a.m;
  const double r = a.res[s];
  if (r == 0.0) return;
  const int2 L = a.lr[s];
  if (L.x > L.y) return;  // no near prism
  const NearBox b = near_box(a.si[s], k);
  const short2* ivs = a.iv + (size_t)s * k.nslots;
  const double xs = a.sxyz[3 * s], ys = a.sxyz[3 * s + 1], zs = a.sxyz[3 * s + 2];
  const int nvx = b.x1 - b.x0 + 2, nvy = b.y1 - b.y0 + 2, nvz = L.y - L.x + 2;
  const int nv = nvx * nvy * nvz;
  if (nv > a.cap) return;  // the host sizes cap for the largest box
  for (int v = lane; v < nv; v += 32) {
    const int ax = b.x0 + v % nvx;
    const int ay = b.y0 + (v / nvx) % nvy;
    const int cz = L.x + v / (nvx * nvy);
    phi[v] = ztm_phi<T>((T)((m.x0 + ax * m.dx) - xs), (T)((m.y0 + ay * m.dy) - ys),
                        (T)((m.zt - cz * m.dz) - zs));
  }
  __syncwarp();
  const int bx = nvx - 1, by = nvy - 1, bz = nvz - 1;
  const int nb = bx * by * bz;
  const long long plane = (long long)m.nx * m.ny;
  for (int q = lane; q < nb; q += 32) {
    const int qx = q % bx, qy = (q / bx) % by, qz = q / (bx * by);
    const int ix = b.x0 + qx, iy = b.y0 + qy, l = L.x + qz;
    const short2 t = ivs[near_slot(b, ix, iy)];
    if (l < t.x || l > t.y) continue;  // not in the near region
    // vertices: x lower qx (-), upper qx+1 (+); z: layer top index qz (+),
    // bottom qz+1 (-)
    auto P = [&](int dx_, int dy_, int dz_) {
      return phi[(qx + dx_) + nvx * ((qy + dy_) + nvy * (qz + dz_))];
    };
    T u = P(1, 1, 0) - P(0, 1, 0) - P(1, 0, 0) + P(0, 0, 0) - P(1, 1, 1) + P(0, 1, 1) + P(1, 0, 1) -
          P(0, 0, 1);
    const long long p = ix + (long long)m.nx * iy + plane * l;
    atomicAdd(&a.g[p], a.G5 * r * (double)u);
  }
  __syncwarp();  // the scratch is rewritten by the warp's next station
}

// Persistent kernel of the mixed adjoint: tiles x slices far items and
// n_near near items (ADJ_NEAR_ST stations, a warp per station) taken from a
// counter, the near items at evenly spaced queue positions.  The grid is the
// number of blocks resident at once.  T: the near regions' type (double for
// the mixed method, float for the FP32 method).
template <typename T>
__global__ void __launch_bounds__(ADJ_TS, 5) adj_kernel(AdjArgs a) {
  __shared__ AdjSmem sm;
  __shared__ int s_item;
  const int n_far = a.tiles * a.slices;
  const int n_items = n_far + a.n_near;
  // queue position i: near iff floor((i+1) n_near / n) > floor(i n_near / n)
  auto near_before = [&](int i) { return (int)((long long)i * a.n_near / n_items); };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* phi = reinterpret_cast<T*>(a.phi + ((size_t)blockIdx.x * (ADJ_TS / 32) + warp) * a.cap);
  for (;;) {
    __syncthreads();  // the previous item is done with s_item and the tiles
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= n_items) break;
    const int nb = near_before(item);
    if (near_before(item + 1) > nb) {
      for (int j = warp; j < ADJ_NEAR_ST; j += ADJ_TS / 32) {
        const int s = nb * ADJ_NEAR_ST + j;
        if (s < a.ns) adj_near_station<T>(a, s, phi, lane);
      }
      continue;
    }
    const int f = item - nb;
    adj_far_item(a, f % a.tiles, f / a.tiles, sm);
  }
}

// ---- plain double ---------------------------------------------------------
// By vertices, as the plain forward: Psi(v) = sum_s resid_s Phi(v - station_s)
// once per mesh vertex (thread per vertex, stations streamed through shared
// memory, per-chunk partials), then g[p] = G * sum over the eight corners of
// p of s_x s_y s_z Psi(corner), s = +1 at the upper and -1 at the lower limit
// of each axis -- the corner form of the prism integral with the station sum
// taken first.  (nx+1)(ny+1)(nz+1) Phi per station instead of 8 nx ny nz.
__global__ void __launch_bounds__(ADJ_TS)
    adj_f64_kernel(MeshDesc m, int ns, const double* __restrict__ sxyz,
                   const double* __restrict__ res, int chunk_len, double* __restrict__ partial) {
  __shared__ double s_st[4 * 128];
  const long long nvx = m.nx + 1, nvy = m.ny + 1, nv = nvx * nvy * (m.nz + 1);
  const long long v = blockIdx.x * (long long)ADJ_TS + threadIdx.x;
  const bool active = v < nv;
  double xv = 0.0, yv = 0.0, zv = 0.0;
  if (active) {
    const int a = (int)(v % nvx), b = (int)((v / nvx) % nvy), c = (int)(v / (nvx * nvy));
    xv = m.x0 + a * m.dx;  // the corner coordinates the corner form uses
    yv = m.y0 + b * m.dy;
    zv = m.zt - c * m.dz;
  }
  const int s0 = blockIdx.y * chunk_len, s1 = min(ns, s0 + chunk_len);
  double acc = 0.0;
  for (int t0 = s0; t0 < s1; t0 += 128) {
    __syncthreads();
    for (int q = threadIdx.x; q < 128; q += ADJ_TS) {
      const int s = t0 + q;
      const bool ok = s < s1;
      s_st[4 * q] = ok ? sxyz[3 * s] : 0.0;
      s_st[4 * q + 1] = ok ? sxyz[3 * s + 1] : 0.0;
      s_st[4 * q + 2] = ok ? sxyz[3 * s + 2] : 0.0;
      s_st[4 * q + 3] = ok ? res[s] : 0.0;
    }
    __syncthreads();
    if (!active) continue;
    const int cnt = min(128, s1 - t0);
    for (int q = 0; q < cnt; q++) {
      const double r = s_st[4 * q + 3];
      if (r == 0.0) continue;
      acc += r * ztm_phi<double>(xv - s_st[4 * q], yv - s_st[4 * q + 1], zv - s_st[4 * q + 2]);
    }
  }
  if (active) partial[(size_t)blockIdx.y * nv + v] = acc;
}

__global__ void adj_f64_finalize(MeshDesc m, int nchunks, const double* __restrict__ partial,
                                 double G5, double* __restrict__ g) {
  const long long np = (long long)m.nx * m.ny * m.nz;
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= np) return;
  const long long nvx = m.nx + 1, nvy = m.ny + 1, nv = nvx * nvy * (m.nz + 1);
  const long long plane = (long long)m.nx * m.ny;
  const int l = (int)(p / plane);
  const long long rem = p - (long long)l * plane;
  const int iy = (int)(rem / m.nx), ix = (int)(rem % m.nx);
  double a = 0.0;
#pragma unroll
  for (int dc = 0; dc < 2; dc++)      // c = l: top (+), c = l + 1: bottom (-)
#pragma unroll
    for (int db = 0; db < 2; db++)    // b = iy: lower (-), b = iy + 1: upper (+)
#pragma unroll
      for (int da = 0; da < 2; da++) {
        const long long v = (ix + da) + nvx * ((iy + db) + nvy * (long long)(l + dc));
        double psi = 0.0;
        for (int c = 0; c < nchunks; c++) psi += partial[(size_t)c * nv + v];
        const bool neg = (da == 0) ^ (db == 0) ^ (dc == 1);
        a += neg ? -psi : psi;
      }
  g[p] = G5 * a;
}

// Station chunks of the plain double adjoint over nv vertices.
int adj_f64_chunks(long long nv, int ns, int num_sms, int* len) {
  long long blocks = (nv + ADJ_TS - 1) / ADJ_TS;
  long long want = std::max(1LL, (8LL * std::max(num_sms, 1)) / std::max(blocks, 1LL));
  long long ch = std::min<long long>(std::min(want, (long long)std::max(1, ns / 32)), 65535);
  ch = std::max(1LL, ch);
  int l = (int)((ns + ch - 1) / ch);
  *len = std::max(l, 1);
  return (ns + *len - 1) / *len;
}

int near_cap(const MeshConst& k) {
  return (std::min(2 * k.wx + 1, k.nx) + 1) * (std::min(2 * k.wy + 1, k.ny) + 1) *
         (std::min(2 * k.wl + 1, k.nz) + 1);
}

// Blocks of the persistent adjoint kernel resident at once (its grid); the
// larger of the two near-region types, which sizes the vertex scratch.
int adj_grid(int num_sms, bool f64) {
  int occ = 0;
  const cudaError_t e =
      f64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adj_kernel<double>, ADJ_TS, 0)
          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adj_kernel<float>, ADJ_TS, 0);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    occ = 1;
  }
  return occ * std::max(num_sms, 1);
}
int adj_grid_max(int num_sms) { return std::max(adj_grid(num_sms, true), adj_grid(num_sms, false)); }

}  // namespace

size_t ztm_adjoint_ws(const MeshDesc& m, int ns, int precision, int num_sms, double near_q) {
  long long np = (long long)m.nx * m.ny * m.nz;
  if (precision == ZTM_PREC_FP64) {
    const long long nv = (long long)(m.nx + 1) * (m.ny + 1) * (m.nz + 1);
    int len;
    int ch = adj_f64_chunks(nv, std::max(ns, 1), num_sms, &len);
    return WsCarver::need((size_t)ch * nv * 8);
  }
  const MeshConst k = make_mesh_const(m, near_q > 0 ? near_q : ZTM_MESH_NEAR_Q);
  return 2 * WsCarver::need((size_t)std::max(ns, 1) * 16) +
         WsCarver::need((size_t)std::max(ns, 1) * k.nslots * 4) +
         WsCarver::need((size_t)std::max(ns, 1) * 8) + WsCarver::need(64) +
         WsCarver::need((size_t)adj_grid_max(num_sms) * (ADJ_TS / 32) * near_cap(k) * 8);
}

int ztm_launch_adjoint(ztm_ctx* c, const MeshDesc& m, int ns, const double* d_sxyz,
                       const double* d_res, double* d_g, double G, int precision,
                       const ztm_opts* o, WsCarver& wc) {
  const double G5 = G * 1.0e5;
  const long long np = (long long)m.nx * m.ny * m.nz;
  if (ns == 0) {
    cudaMemsetAsync(d_g, 0, np * 8, c->stream);
    return ztm_after_launch(c, "adjoint (no stations)");
  }
  if (precision == ZTM_PREC_FP64) {
    const long long nv = (long long)(m.nx + 1) * (m.ny + 1) * (m.nz + 1);
    if (nv > (1LL << 31) - 1) return ztm_fail(c, ZTM_ERR_RANGE, "mesh has more than 2^31-1 vertices");
    int len;
    int ch = adj_f64_chunks(nv, ns, c->num_sms, &len);
    double* partial = wc.take<double>((size_t)ch * nv);
    dim3 grid((unsigned)((nv + ADJ_TS - 1) / ADJ_TS), ch);
    {
      ZtmProf prof_(c, "adjoint_f64");
      adj_f64_kernel<<<grid, ADJ_TS, 0, c->stream>>>(m, ns, d_sxyz, d_res, len, partial);
    }
    adj_f64_finalize<<<(unsigned)((np + 255) / 256), 256, 0, c->stream>>>(m, ch, partial, G5, d_g);
    c->launches += 2;
    return ztm_after_launch(c, "adjoint FP64 kernels");
  }
  const double nq = (o && o->near_q > 0) ? o->near_q : ZTM_MESH_NEAR_Q;
  MeshConst k = make_mesh_const(m, nq);
  if (m.nz > 32767) return ztm_fail(c, ZTM_ERR_RANGE, "mixed adjoint supports nz <= 32767");
  float4* sf = wc.take<float4>(ns);
  int4* si = wc.take<int4>(ns);
  short2* iv = wc.take<short2>((size_t)ns * k.nslots);
  int2* lr = wc.take<int2>(ns);
  launch_mesh_station_prep(c, m, k.L0, ns, d_sxyz, sf, si);
  launch_mesh_near_iv(c, k, m, ns, si, d_sxyz, iv, lr);
  const int ngroups = (k.nz + ADJ_LG - 1) / ADJ_LG;
  const double scale = G5 * k.L0 * (double)k.dxn * k.dyn * k.dzn;
  const int cap = near_cap(k);
  if ((size_t)cap * 8 > 200 * 1024)
    return ztm_fail(c, ZTM_ERR_RANGE, "near_q too large for the adjoint's near box");
  const bool f64 = precision == ZTM_PREC_MIXED;
  // station slices so that there are about sixteen far items per resident
  // block (measured: 4 items 22.2 ms, 8 21.1, 16 20.4, 24 20.8, 32 20.7);
  // the slices' sums meet in g by double atomics (g zeroed first)
  const long long tiles = (long long)((k.ncols + ADJ_TS - 1) / ADJ_TS) * ngroups;
  const int grid = adj_grid(c->num_sms, f64);
  long long slices = std::max(1LL, (16LL * grid + tiles - 1) / tiles);
  slices = std::min(slices, std::max(1LL, (long long)(ns + ADJ_STILE - 1) / ADJ_STILE));
  int slice = (int)((ns + slices - 1) / slices);
  slice = ((slice + ADJ_STILE - 1) / ADJ_STILE) * ADJ_STILE;
  slices = (ns + slice - 1) / slice;
  if (tiles * slices + (ns + ADJ_NEAR_ST - 1) / ADJ_NEAR_ST > 2147483647LL)
    return ztm_fail(c, ZTM_ERR_RANGE, "mixed adjoint: too many work items");
  int* counter = wc.take<int>(16);
  double* phi = wc.take<double>((size_t)adj_grid_max(c->num_sms) * (ADJ_TS / 32) * cap);
  AdjArgs a;
  a.k = k;
  a.m = m;
  a.ns = ns;
  a.sf = sf;
  a.si = si;
  a.iv = iv;
  a.lr = lr;
  a.sxyz = d_sxyz;
  a.res = d_res;
  a.scale = scale;
  a.G5 = G5;
  a.slice = slice;
  a.tiles = (int)tiles;
  a.slices = (int)slices;
  a.n_near = (ns + ADJ_NEAR_ST - 1) / ADJ_NEAR_ST;
  a.cap = cap;
  a.phi = phi;
  a.counter = counter;
  a.g = d_g;
  cudaMemsetAsync(d_g, 0, (size_t)k.ncols * k.nz * sizeof(double), c->stream);
  cudaMemsetAsync(counter, 0, sizeof(int), c->stream);
  // far fields (FMA pipe) and near regions (FP64 pipe) in one persistent grid
  {
    ZtmProf prof_(c, "adjoint_far");
    if (f64)
      adj_kernel<double><<<grid, ADJ_TS, 0, c->stream>>>(a);
    else
      adj_kernel<float><<<grid, ADJ_TS, 0, c->stream>>>(a);
  }
  c->launches += 1;
  return ztm_after_launch(c, "adjoint mixed kernels");
}
