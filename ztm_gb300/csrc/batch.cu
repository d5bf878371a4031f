// batch.cu - batched prism forward: many density models and uneven meshes
// in one persistent launch, replayed from a CUDA graph.
//
// The reference evaluates its damping trials one full forward model after
// another (TFM.cpp:165, each FM call running the GPU process of
// TFM.cpp:90-94).  Here a job is (mesh, stations, nmodels densities); the
// trial models of a line search are one job with nmodels > 1 and share every
// pair's geometry: the far-field kernel value K of a (station, prism) pair is
// computed once and applied to every model of a group, so that the far field
// of the group is a contraction over prisms, sum_p K(s, p) rho_m(p).
// Independent regional meshes are further jobs.
//
// Work items, taken from one global counter by a persistent grid of
// (resident blocks x SMs), the near items spread evenly over the first half
// of the queue (the FP64 pipe busy beside the FMA pipe and the tensor cores):
//   near item  (job, station tile): a warp per station; for one model the
//              forward's vertex pass (near_station), for several Phi at the
//              near-box vertices in double once into the warp's slice of a
//              global scratch, then the unit responses of the near prisms
//              and per model one multiply-add per near prism.
//   far item   (job, station tile, column chunk, model group):
//              - tensor-core variant, multi-model jobs (far_item_tc): 32
//                models per group; each thread evaluates K for its station,
//                splits it into TF32 high part and FP32 remainder in its TMEM
//                lane, and tcgen05 MMAs (A from TMEM, B = the models' split
//                densities, one 1-D bulk copy per column in the MMA's
//                shared-memory layout) accumulate the contraction in TMEM;
//              - CUDA-core variants (far_item_cc): models interleaved in HBM,
//                one bulk copy per stage, packed FMAs into compensated sums;
//              - one-model jobs: the mixed forward's column loop
//                (meshfar::far_stage).
// Every item bumps its tile's completion counter; the block that completes a
// tile adds the tile's partials in a fixed order and writes gz, so the launch
// needs no second kernel and the result is deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "mesh_far.cuh"
#include "prism_common.cuh"
#include "tc_tf32.cuh"
#include "ztm_internal.cuh"

namespace {

constexpr int B_TS = 128;   // threads per block = stations per tile
constexpr int B_WARPS = B_TS / 32;

struct BJob {
  MeshConst k;
  MeshDesc m;
  int nmodels, ns, tiles, chunks, chunk_cols, sc, mgroups, nv_cap;
  int mgw;               // models interleaved per group: 1 or the variant's MG
  int tc, nzt;           // far items on the tensor cores; their layers per column
                         // (nz rounded up to a multiple of 16)
  long long near_base, far_base;
  double far_scale, G5;
  const float4* sf;
  const int4* si;
  const int* perm;       // station of each tile slot (Z order of the home cells)
  const short2* iv;      // near-region intervals [station][box column]
  const int2* lr;        // per-station near layer range
  const float* rhoT;     // [group][column][layer][mgw] float densities
  const float* rhoC;     // tensor-core jobs: [group][column][MMA B layout]
  const double* rho;     // nmodels x np (layer-major, as given)
  const double* sxyz;
  double* partial;       // [model][chunk][ns]
  double* near;          // [model][ns]
  double* gz;            // [model][ns]
  int* done;             // [tiles]
};

struct BArgs {
  const BJob* jobs;
  int njobs;
  long long n_near, n_items;
  long long near_span;  // queue positions the near items are spread over
  int* counter;
  int* err;
  double* phi;   // [block][warp][phi_stride] near-box vertex values and the
                 // near prisms' unit responses (global scratch)
  int phi_cap;
  int phi_stride;  // doubles per warp: 2 phi_cap
  int drain;       // tensor-core items: k-blocks per accumulation window
  unsigned poll_limit;  // test hook, 0 = off: the tensor-core items' stage
                        // waits poll a barrier that nothing completes
};

// Float densities of a job, model-interleaved: rhoT[((g*ncols + c)*nzp + l)*W
// + mm] = rho_{g*W+mm}(c, l), zero for padded layers or models.  A far item's
// stage (a run of columns of one model group) is one contiguous range, and a
// layer's W model densities are adjacent.
__global__ void transpose_models_kernel(MeshConst k, int nmodels, int W,
                                        const double* __restrict__ rho,
                                        float* __restrict__ rhoT) {
  const int ngroups = (nmodels + W - 1) / W;
  const long long total = (long long)ngroups * k.ncols * k.nzp * W;
  const long long np = (long long)k.ncols * k.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int mm = (int)(t % W);
    long long r = t / W;
    const int l = (int)(r % k.nzp);
    r /= k.nzp;
    const int c = (int)(r % k.ncols);
    const int g = (int)(r / k.ncols);
    const int md = g * W + mm;
    float v = 0.f;
    if (l < k.nz && md < nmodels) v = (float)rho[(long long)md * np + (long long)l * k.ncols + c];
    rhoT[t] = v;
  }
}

// Far field of one column for every model of the group, W models
// interleaved in `col` (layer-major, W per layer).  K is computed once per
// (station, prism) pair; two packed FMAs per model pair and layer; plain
// sums over 64 layers, Kahan across groups.
// T2: the second-order form (every lane of the warp far enough); MASK: some
// lane of the warp has the column in its near box, or nz is not a multiple
// of 8 (both warp-uniform, so the selects are skipped for most columns).
// Kahan accumulators of this thread's models in shared memory (model m at
// ks[m * B_TS], kc[m * B_TS]; the pointers are offset by the thread index).
__device__ __forceinline__ void kahan_smem(float* ks, float* kc, int m, float x) {
  const float y = x - kc[m * B_TS];
  const float s0 = ks[m * B_TS];
  const float t = s0 + y;
  kc[m * B_TS] = (t - s0) - y;
  ks[m * B_TS] = t;
}

template <int W, bool T2, bool MASK>
__device__ __forceinline__ void far_column(const float* __restrict__ col, const MeshConst& k,
                                           const ColPoly2& cp2, float2 c2t, float ez, int izs,
                                           int Lm, int elo, unsigned espan, float* ks,
                                           float* kc) {
  const float2 dz2 = make_float2(k.dzn, k.dzn);
  float zf = (float)(-izs);  // (l0 - izs), exact, stepped by 8
  // plain float sums over up to 64 layers per model, compensated across
  static_assert(W % 4 == 0, "models are read four at a time");
  float2 g[W / 2];
#pragma unroll
  for (int m = 0; m < W / 2; m++) g[m] = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int l0 = 0; l0 < k.nz; l0 += 8, zf += 8.f) {
    const float Zg = fmaf(zf, k.dzn, ez);
    const float2 zg2 = make_float2(Zg, Zg);
    float2 K2[4];  // kernel values of layers (l0+2j, l0+2j+1)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const float2 Z = __ffma2_rn(make_float2((float)(2 * j), (float)(2 * j + 1)), dz2, zg2);
      K2[j] = T2 ? far_unit2_t2(Z, cp2, c2t) : far_unit2(Z, cp2);
      if (MASK) {
        const int la = l0 + 2 * j, lb = la + 1;
        // select: a NaN at a near-region prism is dropped
        if ((la < Lm && (unsigned)(la - elo) <= espan) || la >= k.nz) K2[j].x = 0.f;
        if ((lb < Lm && (unsigned)(lb - elo) <= espan) || lb >= k.nz) K2[j].y = 0.f;
      }
    }
    const bool flush = ((l0 >> 3) & 7) == 7 || l0 + 8 >= k.nz;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float Kj = (j & 1) ? K2[j >> 1].y : K2[j >> 1].x;
      const float2 kk = make_float2(Kj, Kj);
      const float* row = col + (l0 + j) * W;
#pragma unroll
      for (int m = 0; m < W / 4; m++) {
        const float4 r4 = *reinterpret_cast<const float4*>(row + 4 * m);
        g[2 * m] = __ffma2_rn(kk, make_float2(r4.x, r4.y), g[2 * m]);
        g[2 * m + 1] = __ffma2_rn(kk, make_float2(r4.z, r4.w), g[2 * m + 1]);
      }
    }
    if (flush) {
#pragma unroll
      for (int m = 0; m < W / 2; m++) {
        kahan_smem(ks, kc, 2 * m, g[m].x);
        kahan_smem(ks, kc, 2 * m + 1, g[m].y);
        g[m] = make_float2(0.f, 0.f);
      }
    }
  }
}

// tile completion: the last item of a tile writes gz for its stations
__device__ void tile_done(const BJob& J, int tile, int expected, int* s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *s_flag = (atomicAdd(&J.done[tile], 1) == expected - 1);
  __syncthreads();
  if (!*s_flag) return;
  __threadfence();
  const int slot = tile * B_TS + threadIdx.x;
  if (slot >= J.ns) return;
  const int s = J.perm[slot];
  for (int md = 0; md < J.nmodels; md++) {
    const double* pp = J.partial + (size_t)md * J.chunks * J.ns;
    double f = 0.0;
    for (int c = 0; c < J.chunks; c++) f += __ldcg(pp + (size_t)c * J.ns + s);
    const double g = J.far_scale * f + __ldcg(J.near + (size_t)md * J.ns + s);
    J.gz[(size_t)md * J.ns + s] = J.G5 * g;
  }
}

// Near regions of a tile's stations, a warp per station: Phi once per
// vertex next to a near-region prism into the warp's scratch, then each near
// prism's unit response U (the signed sum of Phi over its 8 corners, in
// double), then per model sum_p rho_p U_p: one multiply-add per near prism
// and model.
__device__ void near_item(const BJob& J, int tile, double* phi_all, int phi_cap, int phi_stride,
                          int* err) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* phi = phi_all + (size_t)warp * phi_stride;
  double* U = phi + phi_cap;
  if (J.nv_cap > phi_cap) {  // the host sizes phi_cap as the largest nv_cap
    if (threadIdx.x == 0) atomicOr(err, ZTM_DEVERR_BOUNDS);
    return;
  }
  const MeshDesc& m = J.m;
  const long long plane = (long long)m.nx * m.ny;
  const long long np = plane * m.nz;
  for (int j = warp; j < B_TS; j += B_WARPS) {
    const int slot = tile * B_TS + j;
    if (slot >= J.ns) break;
    const int s = J.perm[slot];
    if (J.nmodels == 1) {  // one model: the forward's vertex pass (Phi only where
                           // the region's signed density difference is not zero)
      near_station<double>(J.k, m, s, J.sxyz, J.si, J.iv, J.lr, J.rho, J.near, lane);
      continue;
    }
    const int2 L = J.lr[s];
    if (L.x > L.y) {  // no near prism
      for (int md = lane; md < J.nmodels; md += 32) J.near[(size_t)md * J.ns + s] = 0.0;
      continue;
    }
    const NearBox b = near_box(J.si[s], J.k);
    const short2* ivs = J.iv + (size_t)s * J.k.nslots;
    const double xs = J.sxyz[3 * s], ys = J.sxyz[3 * s + 1], zs = J.sxyz[3 * s + 2];
    const int nvx = b.x1 - b.x0 + 2, nvy = b.y1 - b.y0 + 2, nvz = L.y - L.x + 2;
    const int nv = min(nvx * nvy * nvz, J.nv_cap);
    // is one of the (up to 8) prisms around vertex (a, bb, cz) in the region
    auto touches = [&](int a, int bb, int cz) {
#pragma unroll
      for (int da = 0; da < 2; da++) {
        const int ix = a - 1 + da;
        if (ix < b.x0 || ix > b.x1) continue;
#pragma unroll
        for (int db = 0; db < 2; db++) {
          const int iy = bb - 1 + db;
          if (iy < b.y0 || iy > b.y1) continue;
          const short2 t = ivs[near_slot(b, ix, iy)];
          if (t.x <= t.y && t.x <= cz && cz - 1 <= t.y) return true;  // layer cz - 1 or cz
        }
      }
      return false;
    };
    for (int v = lane; v < nv; v += 32) {
      const int a = b.x0 + v % nvx, bb = b.y0 + (v / nvx) % nvy, cz = L.x + v / (nvx * nvy);
      phi[v] = touches(a, bb, cz) ? ztm_phi<double>((m.x0 + a * m.dx) - xs,
                                                    (m.y0 + bb * m.dy) - ys,
                                                    (m.zt - cz * m.dz) - zs)
                                  : 0.0;
    }
    __syncwarp();
    // unit responses: vertices x lower qx (-), upper qx+1 (+); z: layer top
    // index qz (+), bottom qz+1 (-); zero outside the region
    const int bx = nvx - 1, by = nvy - 1, bz = nvz - 1;
    const int nbp = bx * by * bz;  // < nv
    for (int q = lane; q < nbp; q += 32) {
      const int qx = q % bx, qy = (q / bx) % by, qz = q / (bx * by);
      const short2 t = ivs[near_slot(b, b.x0 + qx, b.y0 + qy)];
      const int l = L.x + qz;
      double u = 0.0;
      if (l >= t.x && l <= t.y) {
        auto P = [&](int dx_, int dy_, int dz_) {
          return phi[(qx + dx_) + nvx * ((qy + dy_) + nvy * (qz + dz_))];
        };
        u = P(1, 1, 0) - P(0, 1, 0) - P(1, 0, 0) + P(0, 0, 0) - P(1, 1, 1) + P(0, 1, 1) +
            P(1, 0, 1) - P(0, 0, 1);
      }
      U[q] = u;
    }
    __syncwarp();
    for (int md = 0; md < J.nmodels; md++) {
      const double* rho = J.rho + (size_t)md * np;
      double acc = 0.0;
      for (int q = lane; q < nbp; q += 32) {
        const double u = U[q];
        if (u == 0.0) continue;
        const int qx = q % bx, qy = (q / bx) % by, qz = q / (bx * by);
        acc = fma(rho[(b.x0 + qx) + (long long)m.nx * (b.y0 + qy) + plane * (L.x + qz)], u, acc);
      }
      acc = warp_sum_d(acc);
      if (lane == 0) J.near[(size_t)md * J.ns + s] = acc;
    }
    __syncwarp();
  }
}

// One far item on the CUDA cores: (job, station tile, column chunk, model
// group of MG, or one model where the job has one: then the mixed forward's
// own column loop, meshfar::far_stage, with its column pairs and
// second-order shortcut).  Returns false if a stage wait ran out (the caller
// reports the timeout).
template <int MG>
__device__ bool far_item_cc(const BJob& J, int tile, int chunk, int mg, uint64_t* bar,
                            float* stage, unsigned& uses0, unsigned& uses1, float* ks,
                            float* kc, int* s_lm) {
  const MeshConst& k = J.k;
  const int m0 = mg * J.mgw, mcnt = min(J.mgw, J.nmodels - m0);
  const int c0 = chunk * J.chunk_cols, c1 = min(k.ncols, c0 + J.chunk_cols);
  const int nst = (c1 - c0 + J.sc - 1) / J.sc;
  const int stage_floats = J.sc * k.nzp * J.mgw;
  const int slot = tile * B_TS + threadIdx.x;
  const bool active = slot < J.ns;
  const int s = active ? J.perm[slot] : 0;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  int ixs = 0, iys = 0, izs = 0;
  NearBox nb = {1, 0, 1, 0, 1, 0};
  if (threadIdx.x == 0) *s_lm = 0;
  __syncthreads();
  if (active) {
    const float4 f = J.sf[s];
    const int4 i = J.si[s];
    ex = f.x; ey = f.y; ez = f.z;
    ixs = i.x; iys = i.y; izs = i.z;
    nb = near_box(i, k);
    atomicMax(s_lm, nb.l1 + 1);
  }
  auto issue = [&](int st) {
    const int buf = st & 1;
    const int cs = c0 + st * J.sc;
    const int ncol = min(J.sc, c1 - cs);
    const uint32_t bytes = (uint32_t)ncol * k.nzp * J.mgw * 4u;
    mbar_expect_tx(&bar[buf], bytes);
    bulk_g2s(stage + buf * stage_floats,
             J.rhoT + ((size_t)mg * k.ncols + cs) * k.nzp * J.mgw, bytes, &bar[buf]);
  };
  if (threadIdx.x == 0 && nst > 0) issue(0);
  __syncthreads();
  const int Lm = min(*s_lm, k.nz);
  const FarCoef fc = k.fc;
  const bool one = MG == 1 || J.mgw == 1;
  const meshfar::FarStation t = {ex, ey, ez, ixs, iys, izs, nb};
  Kahan acc1;  // the one-model sum
#pragma unroll
  for (int md = 0; md < MG; md++) ks[md * B_TS] = kc[md * B_TS] = 0.f;
  for (int st = 0; st < nst; st++) {
    if (threadIdx.x == 0 && st + 1 < nst) issue(st + 1);
    const int buf = st & 1;
    const unsigned par = (buf ? uses1 : uses0) & 1u;
    const bool ok = mbar_wait(&bar[buf], par);
    if (buf) uses1++; else uses0++;
    if (__syncthreads_or(!ok)) return false;
    const float* rs = stage + buf * stage_floats;
    const int cs = c0 + st * J.sc;
    const int ncol = min(J.sc, c1 - cs);
    if (one) {  // every lane (inactive ones on dummy data) for the warp votes
      unsigned cnt[3];
      meshfar::far_stage<false>(J.iv, k, fc, t, s, Lm, rs, cs, ncol, acc1, cnt);
    } else if constexpr (MG > 1) {
      if (active) {
        int ix = cs % k.nx, iy = cs / k.nx;
        for (int q = 0; q < ncol; q++) {
          const float X = fmaf((float)(ixs - ix), k.dxn, ex);
          const float Y = fmaf((float)(iys - iy), k.dyn, ey);
          const ColPoly cp = col_poly(X, Y, fc);
          const bool ncl = ix >= nb.x0 && ix <= nb.x1 && iy >= nb.y0 && iy <= nb.y1;
          int elo = k.nz;
          unsigned espan = 0u;
          if (ncl) {  // the column's near-region layers
            const short2 tv = J.iv[(size_t)s * k.nslots + near_slot(nb, ix, iy)];
            if (tv.x <= tv.y) {
              elo = tv.x;
              espan = (unsigned)(tv.y - tv.x);
            }
          }
          const float* col = rs + q * k.nzp * J.mgw;
          const ColPoly2 cp2 = col_poly2(cp, fc.a1);
          const float2 c2t = make_float2(cp.C2 - fc.h2, cp.C2 - fc.h2);
          // padded layers (l >= nz) need the mask only below the mesh: for a
          // station with izs < nz their Z is at least half a layer, so K is
          // finite there and the zero densities add nothing
          const unsigned am = __activemask();
          const int form = (__all_sync(am, cp.rh >= k.rh_t2) ? 1 : 0) |
                           ((__any_sync(am, ncl || ((k.nz & 7) && izs >= k.nz))) ? 2 : 0);
          switch (form) {
            case 0: far_column<MG, false, false>(col, k, cp2, c2t, ez, izs, Lm, elo, espan, ks, kc); break;
            case 1: far_column<MG, true, false>(col, k, cp2, c2t, ez, izs, Lm, elo, espan, ks, kc); break;
            case 2: far_column<MG, false, true>(col, k, cp2, c2t, ez, izs, Lm, elo, espan, ks, kc); break;
            default: far_column<MG, true, true>(col, k, cp2, c2t, ez, izs, Lm, elo, espan, ks, kc);
          }
          if (++ix == k.nx) {
            ix = 0;
            ++iy;
          }
        }
      }
    }
    __syncthreads();
  }
  if (active && one) {
    J.partial[((size_t)m0 * J.chunks + chunk) * J.ns + s] = acc1.value();
  } else if (active) {
#pragma unroll
    for (int md = 0; md < MG; md++)
      if (md < mcnt)
        J.partial[((size_t)(m0 + md) * J.chunks + chunk) * J.ns + s] =
            (double)ks[md * B_TS] - (double)kc[md * B_TS];
  }
  return true;
}

// MG models per far item (the interleave width of a multi-model job), MINB
// resident blocks per SM asked of the compiler: the CUDA-core kernel
// variants the autotuner tries (BATCH_VARIANTS).
template <int MG, int MINB>
__global__ void __launch_bounds__(B_TS, MINB) batch_kernel(BArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  float* stage = reinterpret_cast<float*>(smem_raw + 128);
  // near-box vertex values: this block's slice of the global scratch
  // (grid x warps x phi_stride doubles, sized from the same grid on the host)
  double* phi = a.phi + (size_t)blockIdx.x * B_WARPS * a.phi_stride;
  __shared__ long long s_item;
  __shared__ int s_flag, s_lm;
  // compensated sums of each thread's models (16 KB): in registers they
  // would cost 32 per thread
  __shared__ float s_ks[MG * B_TS], s_kc[MG * B_TS];
  float* const ks = s_ks + threadIdx.x;
  float* const kc = s_kc + threadIdx.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  unsigned uses0 = 0, uses1 = 0;  // completed phases per buffer (uniform)
  for (long long guard = 0; guard < a.n_items + 1; guard++) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const long long pos = s_item;
    __syncthreads();
    if (pos >= a.n_items) break;
    // queue position pos < near_span: a near item iff floor((pos+1) n_near /
    // near_span) > floor(pos n_near / near_span), so that the near items
    // (double, FP64 pipe) are spread evenly among the first far items (FMA
    // pipe, tensor cores), none late enough to hold up the end of the launch
    const long long nb = pos < a.near_span ? pos * a.n_near / a.near_span : a.n_near;
    const bool is_near = pos < a.near_span && (pos + 1) * a.n_near / a.near_span > nb;
    // near items are numbered 0 .. n_near - 1, far items n_near .. n_items - 1
    const long long item = is_near ? nb : a.n_near + (pos - nb);
    if (is_near) {
      int j = 0;
      while (j + 1 < a.njobs && a.jobs[j + 1].near_base <= item) j++;
      const BJob& J = a.jobs[j];
      const int tile = (int)(item - J.near_base);
      near_item(J, tile, phi, a.phi_cap, a.phi_stride, a.err);
      __syncthreads();
      tile_done(J, tile, J.chunks * J.mgroups + 1, &s_flag);
      continue;
    }
    int j = 0;
    while (j + 1 < a.njobs && a.jobs[j + 1].far_base <= item) j++;
    const BJob& J = a.jobs[j];
    long long r = item - J.far_base;
    const int tile = (int)(r % J.tiles);
    r /= J.tiles;
    const int chunk = (int)(r % J.chunks);
    const int mg = (int)(r / J.chunks);
    if (!far_item_cc<MG>(J, tile, chunk, mg, bar, stage, uses0, uses1, ks, kc, &s_lm)) {
      if (threadIdx.x == 0) atomicOr(a.err, ZTM_DEVERR_TIMEOUT);
      return;
    }
    tile_done(J, tile, J.chunks * J.mgroups + 1, &s_flag);
  }
}

// ---- multi-model far items on the tensor cores ----------------------------
//
// For a job with many models the far field is a contraction: with K[s][p] the
// far-field value of (station s, prism p), gz_far[s][m] = sum_p K[s][p]
// rho_m[p].  A far item of a tensor-core job is (station tile of 128, column
// chunk, group of TC_MG = 32 models): each thread computes K for its station
// as in far_column, 16 layers at a time, and writes them to its TMEM lane as
// TF32 high and low parts (hi = nearest TF32 of K, lo = K - hi); one thread
// issues per 8 layers two MMAs (M 128, K 8)
//   D[:, 0:64]  += A_hi x [B_hi | B_lo]   (N 64: D[:, 0:32] += A_hi B_hi,
//                                          D[:, 32:64] += A_hi B_lo)
//   D[:, 32:64] += A_lo x B_hi            (N 32)
// with B the group's densities split the same way (B_lo is rho - B_hi), so
// D[:, m] + D[:, 32 + m] carries K rho_m to about 2^-22 of each product (the
// dropped lo x lo term and the TF32 rounding of the low parts).  The tensor
// core's FP32 accumulation truncates: every add into an accumulator loses
// about half a unit in its last place, toward zero.  So the main products
// D[:, 0:32] take one add per 8 layers, and every `drain` k-blocks (default
// 4: 8 adds, a bias of about 2e-7 of the window's sum) D is read back
// (tcgen05.ld) and added to the thread's compensated sums in registers; the
// cross products D[:, 32:64] (terms about 2^-11 of the main ones) have their
// own columns.  (Two adds into the main accumulator per 8 layers and 32 per
// window measured 1.6e-6 on the 256x256x64 line search.)
//
// On this tensor core an MMA of N <= 64 costs about 47 cycles of issue for
// K = 8 (N = 256 about 130), and one MMA's issue-to-mbarrier round trip
// about 250 cycles: with four blocks sharing the SM's tensor core, the MMAs
// of a k-block must complete within the next k-block's K evaluation, so
// fewer and wider MMAs (two, not three, per 8 layers) help.  The block is
// sized for occupancy (128 TMEM columns and 128 registers a thread: four
// blocks per SM).
//
// B comes from HBM ready in the MMA's shared-memory layout (see
// transpose_models_tc_kernel), one 1-D bulk copy per column into a ring of
// TC_NS stages, issued one column ahead.  Synchronisation, per block:
//   stage[i]  bulk copy of a column landed (thread 0 waits before its MMAs);
//   mma[b]    tcgen05.commit after the MMAs that read A buffer b: every thread
//             waits for k-block n - 2 before writing buffer n & 1, and the
//             drain waits for the last k-block before reading D.  Waiting for
//             k-block n - 2 also frees the stage of column c - 2 (commits
//             complete in order, and a column has at least one k-block), which
//             is the stage the copy issued at the start of column c fills.
constexpr int TC_MG = 32;           // models per tensor-core group
constexpr int TC_N = 2 * TC_MG;     // rows of B: the high parts, then the low parts
constexpr int TC_NS = 3;            // column stages
constexpr int TC_KB = 16;           // layers per k-block (two MMA steps of K = 8)
constexpr uint32_t TC_COLS = 128;   // TMEM columns: D [0, 64), A buffer b at 64 + 32 b
constexpr uint32_t TC_IDESC = tc_idesc_tf32(128, TC_MG);
constexpr uint32_t TC_IDESC64 = tc_idesc_tf32(128, TC_N);

// Densities of a tensor-core job in the MMA's B layout, one column after
// another: per column, per 8 layers (lb), the two K halves (kc: layers
// +0..3, +4..7) of TC_N rows in groups of 8 (ng), each row 16 bytes (4
// layers): rhoC[((((g ncols + c) (nzt/8) + lb) 2 + kc) (TC_N/8) + ng) 32 +
// nr 4 + kk] = part(n) of rho_{g TC_MG + n % TC_MG}(c, 8 lb + 4 kc + kk),
// n = 8 ng + nr, part 0 (n < TC_MG) the nearest TF32 value h of the density,
// part 1 the nearest TF32 value of (density - h); zero for padded layers and
// models.  A column is one contiguous range (one bulk copy), and 8 layers of
// it are one MMA step's B operand with LBO = TC_N * 16 bytes (kc stride) and
// SBO = 128 bytes (ng stride).
__global__ void __launch_bounds__(256) transpose_models_tc_kernel(MeshConst k, int nmodels,
                                                                    int nzt,
                                                                    const double* __restrict__ rho,
                                                                    float* __restrict__ rhoC) {
  // a block per (model group, 8-layer block lb, 16 consecutive columns): the
  // 32 models x 8 layers x 16 columns are read along the columns (coalesced)
  // into shared memory, then each column's 8-layer block (64 rows x 8 layers,
  // 2 KB, contiguous in rhoC) is written by consecutive threads
  __shared__ double t[TC_MG * 8][17];
  const int nlb = nzt / 8, ncb = (k.ncols + 15) / 16;
  const int ngroups = (nmodels + TC_MG - 1) / TC_MG;
  const long long np = (long long)k.ncols * k.nz;
  const long long nblk = (long long)ngroups * nlb * ncb;
  for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int cb = (int)(blk % ncb);
    const int lb = (int)((blk / ncb) % nlb);
    const int g = (int)(blk / ((long long)ncb * nlb));
    const int c0 = cb * 16;
    __syncthreads();
    for (int e = threadIdx.x; e < TC_MG * 8 * 16; e += 256) {
      const int cc = e & 15, row = e >> 4;  // row = m * 8 + layer within the block
      const int m = row >> 3, l = lb * 8 + (row & 7), md = g * TC_MG + m, c = c0 + cc;
      double v = 0.0;
      if (md < nmodels && l < k.nz && c < k.ncols) v = rho[(long long)md * np + (long long)l * k.ncols + c];
      t[row][cc] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 16 * 8 * TC_N; e += 256) {
      const int cc = e / (8 * TC_N), w = e % (8 * TC_N);  // w: position in the column's block
      const int c = c0 + cc;
      if (c >= k.ncols) continue;
      const int kk = w & 3, nr = (w >> 2) & 7, ng = (w >> 5) % (TC_N / 8), kc = (w >> 5) / (TC_N / 8);
      const int n = ng * 8 + nr, m = n % TC_MG, lw = kc * 4 + kk;
      const double x = t[m * 8 + lw][cc];
      const float h = __uint_as_float(tf32_rna((float)x));
      const float v = n < TC_MG ? h : __uint_as_float(tf32_rna((float)(x - (double)h)));
      rhoC[(((long long)g * k.ncols + c) * nlb + lb) * (8 * TC_N) + w] = v;
    }
  }
}

struct TcBars {
  uint64_t stage[TC_NS];
  uint64_t mma[2];
  uint64_t fin;
  uint64_t never;  // the timeout hook's barrier: nothing arrives on it
};

struct TcState {
  uint32_t tmem;      // TMEM base of the block
  unsigned kblk;      // k-blocks committed by the block (uniform)
  unsigned gcol;      // columns staged by the block (uniform)
  unsigned issued;    // stage copies issued (thread 0)
  unsigned waited;    // stage copies waited for (thread 0)
};

__device__ __forceinline__ void kahan_reg(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// K of 16 layers (l0 .. l0 + 15) of one column for this thread's station,
// split into TF32 high parts and FP32 remainders.
template <bool T2, bool MASK>
__device__ __forceinline__ void tc_kblock(const MeshConst& k, const ColPoly2& cp2, float2 c2t,
                                          float ez, float zf0, int l0, int Lm, int elo,
                                          unsigned espan, uint32_t (&hi)[16],
                                          uint32_t (&lo)[16]) {
  const float2 dz2 = make_float2(k.dzn, k.dzn);
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const float Zg = fmaf(zf0 + 8.f * h, k.dzn, ez);
    const float2 zg2 = make_float2(Zg, Zg);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const float2 Z = __ffma2_rn(make_float2((float)(2 * j), (float)(2 * j + 1)), dz2, zg2);
      float2 K = T2 ? far_unit2_t2(Z, cp2, c2t) : far_unit2(Z, cp2);
      if (MASK) {
        const int la = l0 + 8 * h + 2 * j, lb = la + 1;
        // select: a NaN at a near-region prism is dropped
        if ((la < Lm && (unsigned)(la - elo) <= espan) || la >= k.nz) K.x = 0.f;
        if ((lb < Lm && (unsigned)(lb - elo) <= espan) || lb >= k.nz) K.y = 0.f;
      }
      const uint32_t hx = tf32_round_bits(K.x), hy = tf32_round_bits(K.y);
      const float2 L = __ffma2_rn(make_float2(-1.f, -1.f),
                                  make_float2(__uint_as_float(hx), __uint_as_float(hy)), K);
      hi[8 * h + 2 * j] = hx;
      hi[8 * h + 2 * j + 1] = hy;
      lo[8 * h + 2 * j] = __float_as_uint(L.x);
      lo[8 * h + 2 * j + 1] = __float_as_uint(L.y);
    }
  }
}

// One tensor-core far item.  Returns false if a wait ran out (*s_to set).
__device__ bool far_item_tc(const BJob& J, int tile, int chunk, int mg, TcState& ts,
                            TcBars* tb, float* stage, int* s_to, int* s_lm, int drain,
                            unsigned poll_limit) {
  const MeshConst& k = J.k;
  const int tid = threadIdx.x;
  const uint32_t lane_off = (uint32_t)(32 * (tid >> 5)) << 16;
  const int m0 = mg * TC_MG, mcnt = min(TC_MG, J.nmodels - m0);
  const int c0 = chunk * J.chunk_cols, c1 = min(k.ncols, c0 + J.chunk_cols);
  const int ncol = c1 - c0;
  const int nkb = J.nzt / TC_KB;
  const uint32_t col_floats = (uint32_t)J.nzt * TC_N;
  const uint32_t col_bytes = col_floats * 4u;
  const int slot = tile * B_TS + tid;
  const bool active = slot < J.ns;
  const int s = active ? J.perm[slot] : 0;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  int ixs = 0, iys = 0, izs = 0;
  NearBox nb = {1, 0, 1, 0, 1, 0};
  if (tid == 0) *s_lm = 0;
  __syncthreads();
  if (active) {
    const float4 f = J.sf[s];
    const int4 i = J.si[s];
    ex = f.x; ey = f.y; ez = f.z;
    ixs = i.x; iys = i.y; izs = i.z;
    nb = near_box(i, k);
    atomicMax(s_lm, nb.l1 + 1);
  }
  const unsigned g0 = ts.gcol;
  auto issue = [&](int q) {  // thread 0: column c0 + q into stage (g0 + q) % TC_NS
    const unsigned g = g0 + (unsigned)q;
    uint64_t* bar = &tb->stage[g % TC_NS];
    mbar_expect_tx(bar, col_bytes);
    bulk_g2s(stage + (g % TC_NS) * col_floats,
             J.rhoC + ((size_t)mg * k.ncols + c0 + q) * col_floats, col_bytes, bar);
    ts.issued = g + 1;
  };
  if (tid == 0) issue(0);
  __syncthreads();
  const int Lm = min(*s_lm, k.nz);
  const FarCoef fc = k.fc;
  const uint32_t tmem = ts.tmem;
  float as[TC_MG], ac[TC_MG];
#pragma unroll
  for (int m = 0; m < TC_MG; m++) as[m] = ac[m] = 0.f;
  // add D (main and cross products since the last drain) to the compensated
  // sums, once k-block nl's MMAs (and so all before them) have completed
  auto drain_d = [&](unsigned nl) {
    if (!mbar_wait(&tb->mma[nl & 1u], (nl >> 1) & 1u)) *s_to = 1;
    tc_fence_after();
#pragma unroll
    for (int h = 0; h < TC_MG / 16; h++) {
      uint32_t d0[16], d1[16];
      tmem_ld16(tmem + lane_off + 16 * h, d0);
      tmem_ld16(tmem + lane_off + TC_MG + 16 * h, d1);
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; j++)
        kahan_reg(as[16 * h + j], ac[16 * h + j], __uint_as_float(d0[j]) + __uint_as_float(d1[j]));
    }
  };
  bool pending = false;  // D holds products not yet drained
  int win = 0;           // k-blocks into the current accumulation window
  int ix = c0 % k.nx, iy = c0 / k.nx;
  for (int q = 0; q < ncol; q++) {
    const float X = fmaf((float)(ixs - ix), k.dxn, ex);
    const float Y = fmaf((float)(iys - iy), k.dyn, ey);
    const ColPoly cp = col_poly(X, Y, fc);
    const bool ncl = active && ix >= nb.x0 && ix <= nb.x1 && iy >= nb.y0 && iy <= nb.y1;
    int elo = k.nz;
    unsigned espan = 0u;
    if (ncl) {
      const short2 tv = J.iv[(size_t)s * k.nslots + near_slot(nb, ix, iy)];
      if (tv.x <= tv.y) {
        elo = tv.x;
        espan = (unsigned)(tv.y - tv.x);
      }
    }
    const ColPoly2 cp2 = col_poly2(cp, fc.a1);
    const float2 c2t = make_float2(cp.C2 - fc.h2, cp.C2 - fc.h2);
    const int form =
        (__all_sync(0xffffffffu, !active || cp.rh >= k.rh_t2) ? 1 : 0) |
        (__any_sync(0xffffffffu, ncl || (active && (k.nz & (TC_KB - 1)) && izs >= k.nz)) ? 2 : 0);
    // the column's k-blocks, with the form (a compile-time choice of the
    // expansion order and of the near/pad mask) fixed for the whole column
    auto column = [&](auto t2c, auto maskc) {
      constexpr bool T2 = decltype(t2c)::value, MASK = decltype(maskc)::value;
      const unsigned g = g0 + (unsigned)q, si = g % TC_NS;
      // B of the column's first 8 layers; the k-steps follow 2048 bytes
      // (128 descriptor units) apart, the low parts' rows 512 bytes (32
      // units) after the high parts'
      const uint64_t dcol = tc_smem_desc(smem_u32(stage + si * col_floats), TC_N * 16u, 128u);
      float zf = (float)(-izs);
      for (int kb = 0; kb < nkb; kb++, zf += (float)TC_KB) {
        const unsigned n = ts.kblk, b = n & 1u;
        if (n >= 2) {  // the MMAs that read A buffer b (k-block n - 2) are done
          if (!mbar_wait(&tb->mma[b], ((n >> 1) - 1u) & 1u)) *s_to = 1;
          tc_fence_after();
        }
        if (tid == 0 && kb == 0 && q + 1 < ncol) issue(q + 1);
        uint32_t hi[16], lo[16];
        tc_kblock<T2, MASK>(k, cp2, c2t, ez, zf, kb * TC_KB, Lm, elo, espan, hi, lo);
        // (a thread without a station writes whatever it computed: its TMEM
        // row only reaches its own row of D, which is never read)
        const uint32_t abuf = tmem + 64u + 32u * b;
        tmem_st16(abuf + lane_off, hi);
        tmem_st16(abuf + lane_off + 16u, lo);
        tmem_wait_st();
        if (tid == 0 && kb == 0) {  // this column's densities in shared memory
          // (the test hook waits on a barrier that nothing completes, with a
          // short bound; a copy not waited for is waited for before the
          // block stops)
          const bool landed = poll_limit ? mbar_poll(&tb->never, 0u, poll_limit)
                                         : mbar_wait(&tb->stage[si], (g / TC_NS) & 1u);
          if (landed) ts.waited = g + 1;
          else *s_to = 1;
        }
        const bool first = win == 0;  // the k-block opens an accumulation window
        if (++win == drain) win = 0;
        if (first && pending) drain_d(n - 1u);
        tc_fence_before();
        __syncthreads();
        if (*s_to) return false;
        if (tid == 0) {
          tc_fence_after();
          const uint64_t d = dcol + (uint64_t)(kb * 256);
          tc_mma_ts(tmem, abuf, d, TC_IDESC64, first ? 0u : 1u);
          tc_mma_ts(tmem + TC_MG, abuf + 16u, d, TC_IDESC, 1u);
          tc_mma_ts(tmem, abuf + 8u, d + 128u, TC_IDESC64, 1u);
          tc_mma_ts(tmem + TC_MG, abuf + 24u, d + 128u, TC_IDESC, 1u);
          tc_commit(&tb->mma[b]);
        }
        ts.kblk = n + 1u;
        pending = true;
      }
      return true;
    };
    bool ok;
    switch (form) {
      case 0: ok = column(std::false_type{}, std::false_type{}); break;
      case 1: ok = column(std::true_type{}, std::false_type{}); break;
      case 2: ok = column(std::false_type{}, std::true_type{}); break;
      default: ok = column(std::true_type{}, std::true_type{});
    }
    if (!ok) return false;
    if (++ix == k.nx) {
      ix = 0;
      ++iy;
    }
  }
  ts.gcol = g0 + (unsigned)ncol;
  if (pending) drain_d(ts.kblk - 1u);
  tc_fence_before();
  __syncthreads();  // every thread has read D before the next item overwrites it
  if (*s_to) return false;
  if (active) {
#pragma unroll
    for (int md = 0; md < TC_MG; md++)
      if (md < mcnt)
        J.partial[((size_t)(m0 + md) * J.chunks + chunk) * J.ns + s] =
            (double)as[md] - (double)ac[md];
  }
  return true;
}

// The tensor-core variant: multi-model jobs (J.tc) by far_item_tc, one-model
// jobs by far_item_cc<1>, near items as in batch_kernel.  TMEM (TC_COLS
// columns) is allocated once per block and freed after the block's last item,
// once its MMAs and stage copies have completed.
template <int MINB>
__global__ void __launch_bounds__(B_TS, MINB) batch_tc_kernel(BArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  float* stage = reinterpret_cast<float*>(smem_raw + 128);
  double* phi = a.phi + (size_t)blockIdx.x * B_WARPS * a.phi_stride;
  __shared__ long long s_item;
  __shared__ int s_flag, s_lm, s_to;
  __shared__ float s_ks[B_TS], s_kc[B_TS];
  __shared__ TcBars tb;
  __shared__ uint32_t s_tmem;
  float* const ks = s_ks + threadIdx.x;
  float* const kc = s_kc + threadIdx.x;
  if ((threadIdx.x >> 5) == 0) {
    tmem_alloc(&s_tmem, TC_COLS);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    for (int i = 0; i < TC_NS; i++) mbar_init(&tb.stage[i], 1);
    mbar_init(&tb.mma[0], 1);
    mbar_init(&tb.mma[1], 1);
    mbar_init(&tb.fin, 1);
    mbar_init(&tb.never, 1);
    fence_mbar_init();
    s_to = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  TcState ts{s_tmem, 0u, 0u, 0u, 0u};
  unsigned uses0 = 0, uses1 = 0;
  bool failed = false;
  for (long long guard = 0; guard < a.n_items + 1; guard++) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const long long pos = s_item;
    __syncthreads();
    if (pos >= a.n_items) break;
    // queue position pos < near_span: a near item iff floor((pos+1) n_near /
    // near_span) > floor(pos n_near / near_span), so that the near items
    // (double, FP64 pipe) are spread evenly among the first far items (FMA
    // pipe, tensor cores), none late enough to hold up the end of the launch
    const long long nb = pos < a.near_span ? pos * a.n_near / a.near_span : a.n_near;
    const bool is_near = pos < a.near_span && (pos + 1) * a.n_near / a.near_span > nb;
    // near items are numbered 0 .. n_near - 1, far items n_near .. n_items - 1
    const long long item = is_near ? nb : a.n_near + (pos - nb);
    if (is_near) {
      int j = 0;
      while (j + 1 < a.njobs && a.jobs[j + 1].near_base <= item) j++;
      const BJob& J = a.jobs[j];
      const int tile = (int)(item - J.near_base);
      near_item(J, tile, phi, a.phi_cap, a.phi_stride, a.err);
      __syncthreads();
      tile_done(J, tile, J.chunks * J.mgroups + 1, &s_flag);
      continue;
    }
    int j = 0;
    while (j + 1 < a.njobs && a.jobs[j + 1].far_base <= item) j++;
    const BJob& J = a.jobs[j];
    long long r = item - J.far_base;
    const int tile = (int)(r % J.tiles);
    r /= J.tiles;
    const int chunk = (int)(r % J.chunks);
    const int mg = (int)(r / J.chunks);
    const bool ok = J.tc ? far_item_tc(J, tile, chunk, mg, ts, &tb, stage, &s_to, &s_lm, a.drain,
                                       a.poll_limit)
                         : far_item_cc<1>(J, tile, chunk, mg, bar, stage, uses0, uses1, ks, kc,
                                          &s_lm);
    if (!ok) {
      failed = true;
      break;
    }
    tile_done(J, tile, J.chunks * J.mgroups + 1, &s_flag);
  }
  if (failed && threadIdx.x == 0) atomicOr(a.err, ZTM_DEVERR_TIMEOUT);
  // before TMEM is freed: every MMA of the block complete, every stage copy
  // landed (bounded waits; a wait that runs out only adds to the error)
  if (threadIdx.x == 0) tc_commit(&tb.fin);
  if (!mbar_wait(&tb.fin, 0u) && threadIdx.x == 0) atomicOr(a.err, ZTM_DEVERR_TIMEOUT);
  if (threadIdx.x == 0)
    for (unsigned g = ts.waited; g < ts.issued; g++)
      if (!mbar_wait(&tb.stage[g % TC_NS], (g / TC_NS) & 1u)) atomicOr(a.err, ZTM_DEVERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(ts.tmem, TC_COLS);
}

struct Plan {
  std::vector<BJob> jobs;
  long long n_near = 0, n_items = 0;
  size_t smem = 128;
  size_t ws_bytes = 0;
  int phi_cap = 0;
};

// Shapes only (no pointers): per-job tiles, chunks, stage widths, workspace.
// tc: multi-model jobs take their far items on the tensor cores (one column
// per stage, TC_MG models per group; stage_kb is then unused).
Plan plan(const ztm_job* jobs, int njobs, double near_q, int num_sms, int stage_kb, int tlog2,
          int mg, bool tc) {
  Plan p;
  size_t ws = 0;
  for (int j = 0; j < njobs; j++) {
    const ztm_job& q = jobs[j];
    BJob J;
    MeshDesc m;
    m.nx = q.mesh.nx; m.ny = q.mesh.ny; m.nz = q.mesh.nz;
    m.x0 = q.mesh.x0; m.y0 = q.mesh.y0; m.zt = q.mesh.z_top;
    m.dx = q.mesh.dx; m.dy = q.mesh.dy; m.dz = q.mesh.dz;
    J.m = m;
    J.k = make_mesh_const(m, near_q);
    J.nmodels = q.nmodels;
    J.ns = q.ns;
    J.tiles = std::max(1, (q.ns + B_TS - 1) / B_TS);
    J.tc = (tc && q.nmodels > 1) ? 1 : 0;
    J.nzt = ((m.nz + TC_KB - 1) / TC_KB) * TC_KB;
    J.mgw = J.tc ? TC_MG : (q.nmodels > 1 ? mg : 1);
    J.mgroups = (q.nmodels + J.mgw - 1) / J.mgw;
    int sc = std::max(1, (stage_kb * 1024) / (J.k.nzp * 4 * J.mgw));
    sc = J.tc ? 1 : std::min(sc, 32);
    J.sc = sc;
    // split columns so that a far item holds about 2^tlog2 (station, prism)
    // pairs (each applied to up to 8 models)
    long long pairs_tile = (long long)B_TS * J.k.ncols * m.nz;
    long long target = 1LL << tlog2;
    int chunks = (int)std::max(1LL, std::min<long long>(pairs_tile / target, J.k.ncols / sc));
    chunks = std::max(chunks, 1);
    int cc = (J.k.ncols + chunks - 1) / chunks;
    cc = ((cc + sc - 1) / sc) * sc;
    J.chunk_cols = cc;
    J.chunks = (J.k.ncols + cc - 1) / cc;
    J.nv_cap = (std::min(2 * J.k.wx + 1, m.nx) + 1) * (std::min(2 * J.k.wy + 1, m.ny) + 1) *
               (std::min(2 * J.k.wl + 1, m.nz) + 1);
    J.far_scale = J.k.L0 * (double)J.k.dxn * J.k.dyn * J.k.dzn;
    const size_t col_floats = J.tc ? (size_t)J.nzt * TC_N : (size_t)J.k.nzp * J.mgw;
    p.smem = std::max(p.smem, 128 + (J.tc ? (size_t)TC_NS : (size_t)2 * sc) * col_floats * 4);
    p.phi_cap = std::max(p.phi_cap, J.nv_cap);
    ws += WsCarver::need((size_t)J.mgroups * J.k.ncols * col_floats * 4);
    ws += WsCarver::need((size_t)q.ns * 16) * 2;
    ws += WsCarver::need((size_t)q.nmodels * J.chunks * q.ns * 8);
    ws += WsCarver::need((size_t)q.nmodels * q.ns * 8);
    ws += WsCarver::need((size_t)J.tiles * 4);
    ws += WsCarver::need((size_t)q.ns * 4) + WsCarver::need(ztm_station_order_ws(q.ns, m.nx, m.ny));
    ws += WsCarver::need((size_t)q.ns * J.k.nslots * 4) + WsCarver::need((size_t)q.ns * 8);
    p.jobs.push_back(J);
  }
  for (auto& J : p.jobs) {
    J.near_base = p.n_near;
    p.n_near += J.tiles;
  }
  long long far = p.n_near;
  for (auto& J : p.jobs) {
    J.far_base = far;
    far += (long long)J.tiles * J.chunks * J.mgroups;
  }
  p.n_items = far;
  // tensor-core variant: at least 48 KB of dynamic shared memory per block,
  // so that no more than 512 / TC_COLS = 4 blocks share an SM's TMEM
  if (tc) p.smem = std::max<size_t>(p.smem, 48 * 1024);
  ws += WsCarver::need(sizeof(BJob) * njobs) + WsCarver::need(64);
  p.ws_bytes = ws;
  (void)num_sms;
  return p;
}

void destroy_entry(ZtmGraphEntry& e) {
  if (e.exec) cudaGraphExecDestroy(e.exec);
  if (e.graph) cudaGraphDestroy(e.graph);
  e.exec = nullptr;
  e.graph = nullptr;
}

// Kernel variants: {models per far item, blocks per SM asked of the
// compiler, tensor cores}.  Variants 0-3 run every far item on the CUDA
// cores; variant 4 runs the far items of multi-model jobs on the tensor cores.
constexpr int BATCH_VARIANTS[][3] = {{16, 4, 0}, {16, 5, 0}, {8, 6, 0}, {32, 3, 0}, {TC_MG, 4, 1}};
using BatchFn = void (*)(BArgs);
BatchFn batch_fn(int v) {
  switch (v) {
    case 1: return batch_kernel<16, 5>;
    case 2: return batch_kernel<8, 6>;
    case 3: return batch_kernel<32, 3>;
    case 4: return batch_tc_kernel<4>;
    default: return batch_kernel<16, 4>;
  }
}

// Launch shapes the autotuner tries: {stage KB per model group (for the
// tensor-core variant: k-blocks per TMEM accumulation window), log2 of the
// pairs per far item, kernel variant}.  The first is the default.  CUDA-core
// variant 0 on 32 trial models on the 256x256x64 mesh plus 16 regional
// meshes: 2^23 pairs 223 ms, 2^24 225 ms, 2^25 229 ms, 2^22 223 ms.
constexpr int BATCH_SHAPES[][3] = {{4, 23, 4},  {2, 23, 4},  {4, 21, 4},  {4, 24, 4},
                                   {16, 23, 0}, {8, 24, 0},  {32, 24, 0}, {16, 24, 0},
                                   {16, 25, 0}, {8, 23, 0},  {32, 25, 0}, {16, 23, 1},
                                   {8, 23, 2},  {16, 23, 2}, {32, 23, 3}, {16, 24, 3}};
constexpr int BATCH_CC_SHAPE = 4;  // the CUDA-core variants' default shape

int batch_run(ztm_ctx* c, const ztm_job* jobs, int njobs, bool dev, double G, double nq,
              int stage_kb, int tlog2, int variant);

}  // namespace

extern "C" int ztm_gfm_batch(ztm_ctx* c, const ztm_job* jobs, int njobs, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (njobs < 0 || (njobs > 0 && !jobs)) return ztm_fail(c, ZTM_ERR_ARG, "bad job list");
  if (njobs == 0) return ZTM_OK;
  if (njobs > 4096) return ztm_fail(c, ZTM_ERR_RANGE, "more than 4096 jobs");
  if (o && (o->precision != ZTM_PREC_MIXED ||
            (o->flags & ~(ZTM_FLAG_DEVICE_PTRS | ZTM_FLAG_AUTOTUNE))))
    return ztm_fail(c, ZTM_ERR_ARG, "batched launches run the mixed method only");
  const bool dev = o && (o->flags & ZTM_FLAG_DEVICE_PTRS);
  const bool tune = o && (o->flags & ZTM_FLAG_AUTOTUNE);
  const double G = (o && o->G > 0) ? o->G : 6.67e-11;
  const double nq = (o && o->near_q > 0) ? o->near_q : ZTM_MESH_NEAR_Q;
  for (int j = 0; j < njobs; j++) {
    const ztm_job& q = jobs[j];
    if (q.mesh.nx < 1 || q.mesh.ny < 1 || q.mesh.nz < 1 || !(q.mesh.dx > 0) ||
        !(q.mesh.dy > 0) || !(q.mesh.dz > 0) || q.nmodels < 1 || q.ns < 1 || !q.rho ||
        !q.sxyz || !q.gz)
      return ztm_fail(c, ZTM_ERR_ARG, "bad job " + std::to_string(j));
    if ((long long)q.mesh.nx * q.mesh.ny * q.mesh.nz * q.nmodels > (1LL << 31) - 1)
      return ztm_fail(c, ZTM_ERR_RANGE, "job " + std::to_string(j) + " is too large");
  }
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device) cudaSetDevice(c->device);
  struct Restore {
    int p, d;
    ~Restore() {
      if (p >= 0 && p != d) cudaSetDevice(p);
    }
  } restore{prev, c->device};
  // the shape: cached for these job shapes, else measured (with
  // ZTM_FLAG_AUTOTUNE: each candidate runs the whole batch once, the fastest
  // is kept on the context), else the default
  std::vector<long long> tkey = {2, njobs, (long long)(nq * 1e6)};
  for (int j = 0; j < njobs; j++)
    tkey.insert(tkey.end(), {jobs[j].mesh.nx, jobs[j].mesh.ny, jobs[j].mesh.nz,
                             jobs[j].nmodels, jobs[j].ns});
  auto it = c->tuned.find(tkey);
  int stage_kb = BATCH_SHAPES[0][0], tlog2 = BATCH_SHAPES[0][1], variant = BATCH_SHAPES[0][2];
  if (it != c->tuned.end()) {
    stage_kb = it->second[0];
    tlog2 = it->second[1];
    variant = it->second[2];
  } else if (tune) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (const auto& sh : BATCH_SHAPES) {
      cudaEventRecord(e0, c->stream);
      const int rc = batch_run(c, jobs, njobs, dev, G, nq, sh[0], sh[1], sh[2]);
      cudaEventRecord(e1, c->stream);
      float ms = 0.f;
      if (rc == ZTM_OK && cudaEventSynchronize(e1) == cudaSuccess &&
          cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
        c->tune_log.push_back({sh[0], sh[1], sh[2], (int)(ms * 1000.f)});
        if (ms < best) {
          best = ms;
          stage_kb = sh[0];
          tlog2 = sh[1];
          variant = sh[2];
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->err.clear();  // a candidate that did not fit is not the call's error
    c->tuned[tkey] = {stage_kb, tlog2, variant};
  }
  return batch_run(c, jobs, njobs, dev, G, nq, stage_kb, tlog2, variant);
}

namespace {

// Blocks of kfn that fit on one SM by registers, shared memory, threads and
// the block limit (the runtime's occupancy query, done by hand: for kernels
// that allocate TMEM it answers 1, while the SM runs as many as fit).
int resident_blocks(ztm_ctx* c, BatchFn kfn, int threads, size_t dyn_smem) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kfn) != cudaSuccess) return 1;
  int regs_sm = 65536, smem_sm = 0, thr_sm = 2048, blk_sm = 32, reserved = 1024;
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, c->device);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, c->device);
  cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, c->device);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, c->device);
  const int warps = (threads + 31) / 32;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;  // allocated per warp
  const int by_regs = regs_warp > 0 ? (regs_sm / regs_warp) / warps : blk_sm;
  const size_t smem_blk = dyn_smem + fa.sharedSizeBytes + (size_t)reserved;
  const int by_smem = (int)((size_t)smem_sm / std::max<size_t>(smem_blk, 1));
  const int by_thr = thr_sm / (warps * 32);
  return std::max(1, std::min(std::min(by_regs, by_smem), std::min(by_thr, blk_sm)));
}

int batch_run(ztm_ctx* c, const ztm_job* jobs, int njobs, bool dev, double G, double nq,
              int stage_kb, int tlog2, int variant) {
  const bool tc = BATCH_VARIANTS[variant][2] != 0;
  Plan p = plan(jobs, njobs, nq, c->num_sms, stage_kb, tlog2, BATCH_VARIANTS[variant][0], tc);
  // the tensor-core items stage whole columns (768 bytes a layer in three
  // stages): a mesh too deep for that runs on the CUDA-core default variant
  if (tc && p.smem > 200 * 1024)
    return batch_run(c, jobs, njobs, dev, G, nq, BATCH_SHAPES[BATCH_CC_SHAPE][0],
                     BATCH_SHAPES[BATCH_CC_SHAPE][1], BATCH_SHAPES[BATCH_CC_SHAPE][2]);
  const BatchFn kfn = batch_fn(variant);
  if (p.smem > 200 * 1024) return ztm_fail(c, ZTM_ERR_RANGE, "near box too large for a batch");
  size_t stage_bytes = 0;
  if (!dev)
    for (int j = 0; j < njobs; j++) {
      const ztm_job& q = jobs[j];
      long long np = (long long)q.mesh.nx * q.mesh.ny * q.mesh.nz;
      stage_bytes += WsCarver::need((size_t)q.nmodels * np * 8) +
                     WsCarver::need((size_t)q.ns * 24) +
                     WsCarver::need((size_t)q.nmodels * q.ns * 8);
    }
  // persistent grid: as many blocks as fit on the device at once
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)std::max<size_t>(p.smem, 48 * 1024));
  int per_sm = 0;
  if (tc)  // the occupancy query answers 1 for a kernel that allocates TMEM
    per_sm = std::min<int>(resident_blocks(c, kfn, B_TS, p.smem), 512 / TC_COLS);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, B_TS, p.smem);
  per_sm = std::max(1, per_sm);
  const long long grid = std::min<long long>((long long)per_sm * c->num_sms, p.n_items);
  const int phi_cap = std::max(p.phi_cap, 1);
  const int phi_stride = 2 * phi_cap;
  const size_t phi_elems = (size_t)grid * B_WARPS * phi_stride;
  int rc = ztm_ws_reserve(c, p.ws_bytes + stage_bytes + WsCarver::need(phi_elems * 8) + 8192);
  if (rc) return rc;
  WsCarver wc(c->ws);
  int* counter = wc.take<int>(16);
  BJob* d_jobs = wc.take<BJob>(njobs);
  double* phi = wc.take<double>(phi_elems);
  std::vector<const double*> rho_d(njobs), xyz_d(njobs);
  std::vector<double*> gz_d(njobs);
  std::vector<char*> order_ws(njobs);  // each job's station-sort scratch
  for (int j = 0; j < njobs; j++) {
    const ztm_job& q = jobs[j];
    long long np = (long long)q.mesh.nx * q.mesh.ny * q.mesh.nz;
    if (dev) {
      rho_d[j] = q.rho;
      xyz_d[j] = q.sxyz;
      gz_d[j] = q.gz;
    } else {
      double* r = wc.take<double>((size_t)q.nmodels * np);
      double* x = wc.take<double>((size_t)q.ns * 3);
      double* g = wc.take<double>((size_t)q.nmodels * q.ns);
      const void* tmp;
      if ((rc = ztm_stage_in(c, q.rho, (size_t)q.nmodels * np * 8, false, r, &tmp))) return rc;
      if ((rc = ztm_stage_in(c, q.sxyz, (size_t)q.ns * 24, false, x, &tmp))) return rc;
      rho_d[j] = r;
      xyz_d[j] = x;
      gz_d[j] = g;
    }
  }
  for (int j = 0; j < njobs; j++) {
    BJob& J = p.jobs[j];
    J.rho = rho_d[j];
    J.sxyz = xyz_d[j];
    J.gz = gz_d[j];
    J.G5 = G * 1.0e5;
    float* rhoT = wc.take<float>((size_t)J.mgroups * J.k.ncols *
                                 (J.tc ? (size_t)J.nzt * TC_N : (size_t)J.k.nzp * J.mgw));
    J.rhoT = J.tc ? nullptr : rhoT;
    J.rhoC = J.tc ? rhoT : nullptr;
    float4* sf = wc.take<float4>(J.ns);
    int4* si = wc.take<int4>(J.ns);
    J.sf = sf;
    J.si = si;
    J.partial = wc.take<double>((size_t)J.nmodels * J.chunks * J.ns);
    J.near = wc.take<double>((size_t)J.nmodels * J.ns);
    J.done = wc.take<int>(J.tiles);
    J.perm = wc.take<int>(J.ns);
    J.iv = wc.take<short2>((size_t)J.ns * J.k.nslots);
    J.lr = wc.take<int2>(J.ns);
    order_ws[j] = wc.take<char>(ztm_station_order_ws(J.ns, J.m.nx, J.m.ny));
  }
  // graph key: shapes and every pointer the graph bakes in
  std::vector<long long> key;
  key.push_back(njobs);
  key.push_back((long long)(size_t)c->ws);
  key.push_back((long long)(size_t)c->stream);
  key.push_back((long long)(nq * 1e6));
  key.push_back(stage_kb);
  key.push_back(tlog2);
  key.push_back(variant);
  key.push_back((long long)c->stage_wait_limit);  // the timeout test hook is baked in
  for (int j = 0; j < njobs; j++) {
    const ztm_job& q = jobs[j];
    key.insert(key.end(), {q.mesh.nx, q.mesh.ny, q.mesh.nz, (long long)(q.mesh.dx * 1e3),
                           (long long)(q.mesh.dy * 1e3), (long long)(q.mesh.dz * 1e3),
                           (long long)(q.mesh.x0 * 1e3), (long long)(q.mesh.y0 * 1e3),
                           (long long)(q.mesh.z_top * 1e3), q.nmodels, q.ns,
                           (long long)(size_t)rho_d[j], (long long)(size_t)xyz_d[j],
                           (long long)(size_t)gz_d[j], (long long)(G * 1e20)});
  }
  // The job table lives in the shared workspace, which other calls reuse:
  // upload it on every call, ahead of the graph, in stream order.  The host
  // copy must outlive the asynchronous copy, so keep it on the context.
  c->batch_table.assign(reinterpret_cast<const char*>(p.jobs.data()),
                        reinterpret_cast<const char*>(p.jobs.data()) + sizeof(BJob) * njobs);
  if ((rc = ztm_cuda_check(c, cudaMemcpyAsync(d_jobs, c->batch_table.data(), sizeof(BJob) * njobs,
                                              cudaMemcpyHostToDevice, c->stream),
                           "upload batch table")))
    return rc;
  ZtmGraphEntry* entry = nullptr;
  for (auto& e : c->graphs)
    if (e.key == key) entry = &e;
  if (!entry) {
    if (c->graphs.size() >= 8) {
      destroy_entry(c->graphs.front());
      c->graphs.erase(c->graphs.begin());
    }
    BArgs args;
    args.phi = phi;
    args.phi_cap = phi_cap;
    args.phi_stride = phi_stride;
    args.jobs = d_jobs;
    args.njobs = njobs;
    args.n_near = p.n_near;
    args.n_items = p.n_items;
    args.near_span = std::max<long long>(1, p.n_near + (p.n_items - p.n_near) / 2);
    args.counter = counter;
    args.err = c->d_err;
    args.drain = tc ? std::max(1, stage_kb) : 1;
    args.poll_limit = tc ? c->stage_wait_limit : 0u;
    ZtmGraphEntry e;
    e.key = key;
    cudaGraph_t g = nullptr;
    const long long launches_before = c->launches;
    if ((rc = ztm_cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal),
                             "begin graph capture")))
      return rc;
    for (int j = 0; j < njobs; j++) {
      BJob& J = p.jobs[j];
      if (J.tc) {
        const long long nblk = (long long)J.mgroups * (J.nzt / 8) * ((J.k.ncols + 15) / 16);
        const int blocks = (int)std::min<long long>(nblk, 16LL * c->num_sms);
        transpose_models_tc_kernel<<<std::max(blocks, 1), 256, 0, c->stream>>>(
            J.k, J.nmodels, J.nzt, J.rho, const_cast<float*>(J.rhoC));
      } else {
        const long long total = (long long)J.mgroups * J.mgw * J.k.ncols * J.k.nzp;
        const int blocks = (int)std::min<long long>((total + 255) / 256, 32LL * c->num_sms);
        transpose_models_kernel<<<std::max(blocks, 1), 256, 0, c->stream>>>(
            J.k, J.nmodels, J.mgw, J.rho, const_cast<float*>(J.rhoT));
      }
      launch_mesh_station_prep(c, J.m, J.k.L0, J.ns, J.sxyz, const_cast<float4*>(J.sf),
                               const_cast<int4*>(J.si));
      WsCarver ow(order_ws[j]);
      if (!rc)
        rc = ztm_station_order(c, c->stream, J.ns, reinterpret_cast<const int*>(J.si), 4, J.m.nx,
                               J.m.ny, const_cast<int*>(J.perm), ow);
      launch_mesh_near_iv(c, J.k, J.m, J.ns, J.si, J.sxyz, const_cast<short2*>(J.iv),
                          const_cast<int2*>(J.lr));
      cudaMemsetAsync(J.done, 0, sizeof(int) * J.tiles, c->stream);
    }
    cudaMemsetAsync(counter, 0, sizeof(int) * 16, c->stream);
    kfn<<<(unsigned)grid, B_TS, p.smem, c->stream>>>(args);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    c->launches = launches_before;  // captured launches are counted per replay
    if (ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return ztm_cuda_check(c, ce, "end graph capture");
    }
    if (rc) {  // a station sort failed to enqueue
      cudaGraphDestroy(g);
      return rc;
    }
    e.graph = g;
    if ((rc = ztm_cuda_check(c, cudaGraphInstantiate(&e.exec, g, 0), "instantiate batch graph"))) {
      cudaGraphDestroy(g);
      return rc;
    }
    c->graphs.push_back(e);
    entry = &c->graphs.back();
  }
  {
    ZtmProf prof_(c, "batch");
    rc = ztm_cuda_check(c, cudaGraphLaunch(entry->exec, c->stream), "launch batch graph");
  }
  if (rc) return rc;
  c->launches += 1 + 4LL * njobs;  // per job: transpose, station prep, sort key, near intervals
  if (dev) return ZTM_OK;
  for (int j = 0; j < njobs; j++) {
    const ztm_job& q = jobs[j];
    if ((rc = ztm_cuda_check(c, cudaMemcpyAsync(q.gz, gz_d[j], (size_t)q.nmodels * q.ns * 8,
                                                cudaMemcpyDeviceToHost, c->stream),
                             "copy batch result")))
      return rc;
  }
  if ((rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "batch"))) return rc;
  return ztm_check_device_error(c);
}

}  // namespace
