// prism.cu - closed-form rectangular-prism gravity forward on sm_103a.
//
// gz(s) = G * 1e5 * sum_p rho_p * U(s, p)   [mGal],
// U(s, p) = integral over prism p of (z_s - z)/r^3 dV
//         = sum over the 8 corners of s_x s_y s_z Phi(corner - station)
// (Nagy 1966; Plouff 1976; Nagy, Papp & Benedek 2000).  The reference has no
// prism model: its gravity path (TFM.cpp:96-98, GFM_GPU.cu:22) is the
// point-mass approximation that the first term of the far-field expansion
// below reproduces.
//
// Three methods:
//   FP64 plain  every pair with the 8-corner closed form in double, the
//               corner function taken once per mesh vertex and station
//               (vertex sharing).  One thread per station, vertices streamed
//               through shared memory, per-chunk partials reduced in a fixed
//               order.
//   MIXED       pairs outside a station's near region (every prism whose
//               centre is >= near_q half-diagonals away, 4 by default) use
//               the sixth-order far-field expansion in float (second order
//               beyond 48 half-diagonals), two layers per packed
//               instruction and two neighbouring columns per pass where the
//               warp allows it, Kahan-summed per thread; the near region is summed in double
//               with vertex sharing (one Phi per vertex instead of 8 per
//               prism); partials and the final per-station sum are double.
//               Stations are taken in Z order of their home cells.  The
//               density of a block's columns is staged in shared memory by
//               1-D TMA bulk copies, double buffered on mbarriers.
//   FP32        as MIXED with the near box also in float.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "mesh_far.cuh"
#include "prism_common.cuh"
#include "ztm_internal.cuh"

namespace {

constexpr int FAR_TS = 128;   // stations per block in the far kernel
constexpr int F64_TS = 64;    // stations per block in the plain double kernel
constexpr int FAR_NEAR_ST = 32;  // stations per near item of the far kernel's queue

// ---------------------------------------------------------------------------
__global__ void station_prep_kernel(MeshDesc m, double L0, int ns,
                                    const double* __restrict__ sxyz,
                                    float4* __restrict__ sf, int4* __restrict__ si) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  const double lim = 1.0e9;
  double fx = fmin(fmax(floor((xs - m.x0) / m.dx), -lim), lim);
  double fy = fmin(fmax(floor((ys - m.y0) / m.dy), -lim), lim);
  double fz = fmin(fmax(floor((m.zt - zs) / m.dz), -lim), lim);
  int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  double ex = (xs - m.x0) - (ix + 0.5) * m.dx;
  double ey = (ys - m.y0) - (iy + 0.5) * m.dy;
  double ez = zs - (m.zt - (iz + 0.5) * m.dz);
  sf[s] = make_float4((float)(ex / L0), (float)(ey / L0), (float)(ez / L0), 0.f);
  si[s] = make_int4(ix, iy, iz, 0);
}

__global__ void transpose_kernel(MeshConst k, int nmodels, const double* __restrict__ rho,
                                 float* __restrict__ rhoT) {
  long long total = (long long)nmodels * k.ncols * k.nzp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long mdl = t / ((long long)k.ncols * k.nzp);
    long long r = t - mdl * (long long)k.ncols * k.nzp;
    int c = (int)(r / k.nzp), l = (int)(r % k.nzp);
    float v = 0.f;
    if (l < k.nz) v = (float)rho[mdl * (long long)k.ncols * k.nz + (long long)l * k.ncols + c];
    rhoT[t] = v;
  }
}

// Near-region intervals of every (station, box column), in double: one
// block per station, a thread per box column; the station's overall layer
// range by shared-memory min/max.  A prism is near when the distance from the
// station to its centre is under near_q half-diagonals (exact coordinates;
// every such prism lies in the near box).
constexpr int NEAR_IV_TS = 128;
__global__ void __launch_bounds__(NEAR_IV_TS)
    near_iv_kernel(MeshConst k, MeshDesc m, int ns, const int4* __restrict__ si,
                   const double* __restrict__ sxyz, short2* __restrict__ iv,
                   int2* __restrict__ lr) {
  __shared__ int s_min, s_max;
  const int s = blockIdx.x;
  if (s >= ns) return;  // uniform over the block
  if (threadIdx.x == 0) {
    s_min = 1 << 30;
    s_max = -1;
  }
  __syncthreads();
  const int4 h = si[s];
  const NearBox b = near_box(h, k);
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  const int bw = b.x1 - b.x0 + 1, bh = b.y1 - b.y0 + 1;
  int lmin = 1 << 30, lmax = -1;
  for (int slot = threadIdx.x; slot < k.nslots; slot += NEAR_IV_TS) {
    short2 out = make_short2(1, 0);
    if (slot < bw * bh) {
      const int ix = b.x0 + slot % bw, iy = b.y0 + slot / bw;
      const double hx = (m.x0 + (ix + 0.5) * m.dx) - xs;
      const double hy = (m.y0 + (iy + 0.5) * m.dy) - ys;
      const double h2 = hx * hx + hy * hy;
      // the predicate, in double; its layers form one interval holding the
      // layer lc nearest the station's height (the distance is convex in l)
      auto in = [&](int l) {
        const double hz = (m.zt - (l + 0.5) * m.dz) - zs;
        return h2 + hz * hz < k.R2;
      };
      const int lc = clampi((int)floor((m.zt - zs) / m.dz), b.l0, b.l1);
      int lo = 1 << 30, hi = -1;
      if (in(lc)) {
        // the interval's ends located in float, then settled in double
        const float h2f = (float)h2, r2f = (float)k.R2, czf = (float)(m.zt - zs),
                    dzf = (float)m.dz;
        int flo = lc, fhi = lc;
        for (int l = b.l0; l <= b.l1; l++) {
          const float hz = fmaf(-((float)l + 0.5f), dzf, czf);
          if (fmaf(hz, hz, h2f) < r2f) {
            flo = min(flo, l);
            fhi = max(fhi, l);
          }
        }
        lo = flo;
        hi = fhi;
        while (lo < lc && !in(lo)) lo++;
        while (lo > b.l0 && in(lo - 1)) lo--;
        while (hi > lc && !in(hi)) hi--;
        while (hi < b.l1 && in(hi + 1)) hi++;
      }
      if (hi >= 0) {
        out = make_short2((short)lo, (short)hi);
        lmin = min(lmin, lo);
        lmax = max(lmax, hi);
      }
    }
    iv[(size_t)s * k.nslots + slot] = out;
  }
  if (lmax >= 0) {
    atomicMin(&s_min, lmin);
    atomicMax(&s_max, lmax);
  }
  __syncthreads();
  if (threadIdx.x == 0) lr[s] = (s_max >= 0) ? make_int2(s_min, s_max) : make_int2(1, 0);
}

// ---------------------------------------------------------------------------
// far field, float, TMA-staged density
struct FarArgs {
  MeshConst k;
  int ns;
  int tiles, chunks;  // work items: tiles x chunks
  int chunk_cols;     // columns per item
  int sc;             // columns per shared-memory stage
  int* counter;       // next work item (zeroed before the launch)
  int n_near;         // near items (FAR_NEAR_ST stations each), spread through the queue
  bool near_f64;      // near region in double (mixed) or float (FP32 method)
  MeshDesc m;
  const double* sxyz;
  const double* rho;  // caller's double density (near region)
  const int2* lr;     // per-station near layer range
  double* near;       // [ns] near-region sums
  const float4* sf;
  const int4* si;
  const short2* iv;  // near-region intervals [station][box column]
  const int* perm;   // station of each tile slot (Z order of the home cells)
  const float* rhoT;
  double* partial;  // [chunk][ns]
  int* err;
  unsigned poll_limit;        // test hook, 0 = off: each stage wait polls a barrier
                              // that nothing completes this many times and gives up
  unsigned long long* forms;  // counting variant: the four form counters
};

__device__ __forceinline__ float far_pair(float rho, float Z, float rh, float a0, float h0,
                                          float h1, const FarCoef& f) {
  const float Z2 = Z * Z;
  const float rinv = rsqrtf(rh + Z2);
  const float ri2 = rinv * rinv;
  const float ri4 = ri2 * ri2;
  const float n2 = fmaf(f.a1, Z2, a0);
  const float H = fmaf(fmaf(f.h2, Z2, h1), Z2, h0);
  const float t = fmaf(H, ri4, n2) * ri4;
  const float base = Z * rinv * ri2 * rho;
  return fmaf(base, t, base);
}

// Persistent kernel of the mixed forward.  The work is tiles x chunks far
// items (a tile of FAR_TS stations against a chunk of chunk_cols columns) and
// n_near near items (the double near regions of FAR_NEAR_ST stations, one
// warp per station), spread evenly through one queue so that while some
// blocks of an SM sum near regions on the FP64 pipe the others sum far
// fields on the FMA pipe.  The grid is the number of blocks resident at once;
// each block takes items from a counter until none are left.  Each far item
// writes its own partial sums (partial[chunk][s]) and each near item its
// stations' near[s], so the result does not depend on which block ran what.
// The density of a far item's columns streams through two shared-memory
// stages by 1-D bulk copies; the next far item's first stage is copied while
// the current item's last stage (or a near item) is processed.
// COUNT: the counting variant (ztm_ctx_count_forms): the same work, with the
// evaluated slots of each form (and the near regions' Phi evaluations) added
// to a.forms at the end.
template <bool COUNT>
__global__ void __launch_bounds__(FAR_TS, 6) far_kernel(FarArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  float* stage = reinterpret_cast<float*>(smem_raw + 128);
  __shared__ int s_lm;
  __shared__ int s_item[2];
  __shared__ int s_to[2];    // a copy wait gave up (by stage parity)
  __shared__ int s_poll[2];  // test hook: thread 0 saw the stage land (by stage parity)
  const MeshConst& k = a.k;
  const int stage_floats = a.sc * k.nzp;
  const int n_far = a.tiles * a.chunks;
  const int n_items = n_far + a.n_near;
  const FarCoef fc = k.fc;

  // queue position i: near iff floor((i+1) n_near / n) > floor(i n_near / n);
  // floor(i n_near / n) near positions come before it
  auto near_before = [&](int i) { return (int)((long long)i * a.n_near / n_items); };
  auto is_near = [&](int i) { return near_before(i + 1) > near_before(i); };
  auto far_index = [&](int i) { return i - near_before(i); };
  // columns [cs, cs + ncol) of stage st of far item f
  auto stage_cols = [&](int f, int st, int* cs) {
    const int c0 = (f / a.tiles) * a.chunk_cols;
    const int c1 = min(k.ncols, c0 + a.chunk_cols);
    *cs = c0 + st * a.sc;
    return min(a.sc, c1 - *cs);
  };
  auto n_stages = [&](int f) {
    const int c0 = (f / a.tiles) * a.chunk_cols;
    const int c1 = min(k.ncols, c0 + a.chunk_cols);
    return (c1 - c0 + a.sc - 1) / a.sc;
  };
  // thread 0 only: copy stage st of far item f into buffer (q & 1)
  auto issue = [&](int f, int st, int q) {
    int cs;
    const int ncol = stage_cols(f, st, &cs);
    const uint32_t bytes = (uint32_t)ncol * k.nzp * 4u;
    mbar_expect_tx(&bar[q & 1], bytes);
    bulk_g2s(stage + (q & 1) * stage_floats, a.rhoT + (size_t)cs * k.nzp, bytes, &bar[q & 1]);
  };

  if (threadIdx.x == 0) {
    s_to[0] = s_to[1] = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);  // the timeout hook's barrier: nothing ever arrives on it
    fence_mbar_init();
    const int first = atomicAdd(a.counter, 1);
    s_item[0] = first;
    s_item[1] = first < n_items ? atomicAdd(a.counter, 1) : n_items;
  }
  __syncthreads();

  int seq = 0;     // stages waited for so far (buffer seq & 1, parity (seq >> 1) & 1)
  int issued = 0;  // stages issued so far (thread 0 issues; every thread keeps the count)
  bool timed_out = false;
  int par = 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned cnt[3] = {0u, 0u, 0u}, nphi = 0u;
  for (;;) {
    const int item = s_item[par];
    if (item >= n_items) break;
    const int nxt = s_item[par ^ 1];
    const bool nxt_far = nxt < n_items && !is_near(nxt);
    if (is_near(item)) {
      // copy the next far item's first stage meanwhile
      if (issued == seq && nxt_far) {
        if (threadIdx.x == 0) issue(far_index(nxt), 0, seq);
        issued = seq + 1;
      }
      const int s0 = near_before(item) * FAR_NEAR_ST;
      for (int j = warp; j < FAR_NEAR_ST; j += FAR_TS / 32) {
        const int s = s0 + j;
        if (s >= a.ns) break;
        if (a.near_f64)
          near_station<double>(k, a.m, s, a.sxyz, a.si, a.iv, a.lr, a.rho, a.near, lane,
                               COUNT ? &nphi : nullptr);
        else
          near_station<float>(k, a.m, s, a.sxyz, a.si, a.iv, a.lr, a.rho, a.near, lane,
                              COUNT ? &nphi : nullptr);
      }
      if (threadIdx.x == 0) s_item[par] = nxt < n_items ? atomicAdd(a.counter, 1) : n_items;
      __syncthreads();
      par ^= 1;
      continue;
    }
    const int f = far_index(item);
    const int tile = f % a.tiles, chunk = f / a.tiles;
    const int slot = tile * FAR_TS + threadIdx.x;
    const bool active = slot < a.ns;
    const int s = active ? a.perm[slot] : 0;
    meshfar::FarStation t = {0.f, 0.f, 0.f, 0, 0, 0, {1, 0, 1, 0, 1, 0}};
    if (active) {
      const float4 fv = a.sf[s];
      const int4 i = a.si[s];
      t.ex = fv.x; t.ey = fv.y; t.ez = fv.z;
      t.ixs = i.x; t.iys = i.y; t.izs = i.z;
      t.nb = near_box(i, k);
    }
    if (threadIdx.x == 0) {
      s_lm = 0;
      if (issued == seq) issue(f, 0, seq);  // not prefetched
    }
    if (issued == seq) issued = seq + 1;
    __syncthreads();
    if (active) atomicMax(&s_lm, t.nb.l1 + 1);
    __syncthreads();
    const int Lm = min(s_lm, k.nz);
    Kahan acc;
    const int nst = n_stages(f);
    for (int st = 0; st < nst; st++) {
      if (threadIdx.x == 0) {
        if (st + 1 < nst)
          issue(f, st + 1, seq + 1);
        else if (nxt_far)
          issue(far_index(nxt), 0, seq + 1);
      }
      if (st + 1 < nst || nxt_far) issued = seq + 2;
      // a thread that gives up on the copy raises the stage's flag and skips
      // the stage; the block leaves together after the stage's barrier (the
      // flags alternate by stage, so a flag raised in the next stage cannot
      // be read by a thread still finishing this one)
      bool landed;
      if (a.poll_limit) {
        // test hook of the timeout path: thread 0 waits, with a short bound,
        // on a barrier that no copy completes, so the wait runs out; one
        // verdict for the whole block, so that no warp splits around the
        // stage's votes.  The copies in flight are waited for below.
        if (threadIdx.x == 0) s_poll[seq & 1] = mbar_poll(&bar[2], 0, a.poll_limit);
        __syncthreads();
        landed = s_poll[seq & 1] && mbar_wait(&bar[seq & 1], (seq >> 1) & 1);
      } else {
        landed = mbar_wait(&bar[seq & 1], (seq >> 1) & 1);
      }
      if (landed) {
        int cs;
        const int ncol = stage_cols(f, st, &cs);
        unsigned c3[3] = {0u, 0u, 0u};
        meshfar::far_stage<COUNT>(a.iv, k, fc, t, s, Lm, stage + (seq & 1) * stage_floats, cs,
                                  ncol, acc, c3);
        if (COUNT && active) {
          cnt[0] += c3[0];
          cnt[1] += c3[1];
          cnt[2] += c3[2];
        }
      } else {
        s_to[seq & 1] = 1;
      }
      __syncthreads();
      if (s_to[seq & 1]) {
        timed_out = true;
        break;
      }
      seq++;
    }
    if (timed_out) break;
    if (active) a.partial[(size_t)chunk * a.ns + s] = acc.value();
    // the next item is s_item[par ^ 1]; refill s_item[par] for the one after
    if (threadIdx.x == 0) s_item[par] = nxt < n_items ? atomicAdd(a.counter, 1) : n_items;
    __syncthreads();
    par ^= 1;
  }
  if (timed_out && threadIdx.x == 0) {
    atomicOr(a.err, ZTM_DEVERR_TIMEOUT);
    // let copies already in flight land before the block's shared memory is
    // released (bounded by the full limit, whatever a.poll_limit says)
    for (int q = seq; q < issued; q++) mbar_wait(&bar[q & 1], (q >> 1) & 1);
  }
  if (COUNT) {
    unsigned long long v[4] = {cnt[0], cnt[1], cnt[2], nphi};
#pragma unroll
    for (int j = 0; j < 4; j++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
      if (lane == 0 && v[j]) atomicAdd(&a.forms[j], v[j]);
    }
  }
}

// gz[s] = G5 * (far_scale * sum_c partial[c][s] + near[s])
__global__ void finalize_kernel(int ns, int nchunks, const double* __restrict__ partial,
                                double far_scale, const double* __restrict__ near,
                                double G5, double* __restrict__ gz) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  double f = 0.0;
  for (int c = 0; c < nchunks; c++) f += partial[(size_t)c * ns + s];
  double g = far_scale * f;
  if (near) g += near[s];
  gz[s] = G5 * g;
}

// ---------------------------------------------------------------------------
// plain double, every pair with the closed form, by vertices.
//
// sum_p rho_p * sum_{corners of p} s_x s_y s_z Phi(corner - station) takes
// each mesh vertex's Phi once per station: gz = sum_v D(v) Phi(v - station),
// with D(v) the sum over the (up to) eight prisms around v of rho_p times
// s_x s_y s_z, s = +1 where v is the prism's upper limit along that axis and
// -1 where it is the lower.  (nx+1)(ny+1)(nz+1) Phi per station instead of
// 8 nx ny nz; each Phi is evaluated at the same double coordinates as the
// corner form evaluates it.  D is formed once per call (vertex_weight_kernel).
__global__ void vertex_weight_kernel(MeshDesc m, const double* __restrict__ rho,
                                     double* __restrict__ D) {
  const long long nvx = m.nx + 1, nvy = m.ny + 1, nv = nvx * nvy * (m.nz + 1);
  const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int a = (int)(v % nvx), b = (int)((v / nvx) % nvy), c = (int)(v / (nvx * nvy));
  const long long plane = (long long)m.nx * m.ny;
  double d = 0.0;
#pragma unroll
  for (int dc = 0; dc < 2; dc++) {
    const int l = c - 1 + dc;  // l = c - 1: v is its bottom (-); l = c: its top (+)
    if (l < 0 || l >= m.nz) continue;
#pragma unroll
    for (int db = 0; db < 2; db++) {
      const int iy = b - 1 + db;  // iy = b - 1: v is its upper y limit (+)
      if (iy < 0 || iy >= m.ny) continue;
#pragma unroll
      for (int da = 0; da < 2; da++) {
        const int ix = a - 1 + da;
        if (ix < 0 || ix >= m.nx) continue;
        const double r = rho[ix + (long long)m.nx * iy + plane * l];
        const bool neg = (da == 1) ^ (db == 1) ^ (dc == 0);
        d += neg ? -r : r;
      }
    }
  }
  D[v] = d;
}

struct __align__(16) Vtx {
  double x, y, z, d;
};

__global__ void __launch_bounds__(F64_TS)
    mesh_f64_kernel(MeshDesc m, int ns, const double* __restrict__ sxyz,
                    const double* __restrict__ D, long long chunk_len,
                    double* __restrict__ partial) {
  __shared__ Vtx tile[256];
  const int s = blockIdx.x * F64_TS + threadIdx.x;
  const bool active = s < ns;
  double xs = 0, ys = 0, zs = 0;
  if (active) {
    xs = sxyz[3 * s];
    ys = sxyz[3 * s + 1];
    zs = sxyz[3 * s + 2];
  }
  const long long nvx = m.nx + 1, nvy = m.ny + 1, nv = nvx * nvy * (m.nz + 1);
  const long long v0 = (long long)blockIdx.y * chunk_len;
  const long long v1 = min(nv, v0 + chunk_len);
  double acc = 0.0;
  for (long long t0 = v0; t0 < v1; t0 += 256) {
    __syncthreads();
    for (int q = threadIdx.x; q < 256; q += F64_TS) {
      const long long v = t0 + q;
      Vtx w = {0.0, 0.0, 0.0, 0.0};
      if (v < v1) {
        const int a = (int)(v % nvx), b = (int)((v / nvx) % nvy), c = (int)(v / (nvx * nvy));
        // corner minus station as the corner form writes it: (x0 + a dx) - xs
        w.x = m.x0 + a * m.dx;
        w.y = m.y0 + b * m.dy;
        w.z = m.zt - c * m.dz;
        w.d = D[v];
      }
      tile[q] = w;
    }
    __syncthreads();
    const int cnt = (int)min(256LL, v1 - t0);
    if (!active) continue;
    for (int q = 0; q < cnt; q++) {
      const Vtx w = tile[q];
      if (w.d == 0.0) continue;  // uniform: all lanes read vertex q
      acc += w.d * ztm_phi<double>(w.x - xs, w.y - ys, w.z - zs);
    }
  }
  if (active) partial[(size_t)blockIdx.y * ns + s] = acc;
}

// ---------------------------------------------------------------------------
// explicit prism lists
struct ListPrism {
  float xh, xl, yh, yl, zh, zl;  // centre (units of 1 km), hi + lo
  float w;                       // rho * volume (km^3)
  float ell2;                    // (near_q * half diagonal)^2 (km^2)
  FarCoef fc;
};

__device__ __forceinline__ void split2(double v, float* h, float* l) {
  float hi = (float)v;
  *h = hi;
  *l = (float)(v - (double)hi);
}

constexpr double LIST_L0 = 1000.0;

__global__ void list_prep_kernel(long long np, const double* __restrict__ geom,
                                 const double* __restrict__ rho, double near_q,
                                 ListPrism* __restrict__ lp) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= np) return;
  const double* g = geom + 6 * q;
  double dx = fabs(g[1] - g[0]), dy = fabs(g[3] - g[2]), dz = fabs(g[5] - g[4]);
  // signed volume: reversed bounds flip the sign, as the closed form does
  double vol = (g[1] - g[0]) * (g[3] - g[2]) * (g[5] - g[4]);
  ListPrism p;
  split2(0.5 * (g[0] + g[1]) / LIST_L0, &p.xh, &p.xl);
  split2(0.5 * (g[2] + g[3]) / LIST_L0, &p.yh, &p.yl);
  split2(0.5 * (g[4] + g[5]) / LIST_L0, &p.zh, &p.zl);
  p.w = (float)(rho[q] * vol / (LIST_L0 * LIST_L0 * LIST_L0));
  double ell = 0.5 * sqrt(dx * dx + dy * dy + dz * dz) / LIST_L0;
  p.ell2 = (float)(near_q * near_q * ell * ell);
  p.fc = far_coef(dx / LIST_L0, dy / LIST_L0, dz / LIST_L0);
  lp[q] = p;
}

template <bool F64NEAR>
__global__ void __launch_bounds__(F64_TS)
    list_kernel(long long np, const double* __restrict__ geom, const double* __restrict__ rho,
                const ListPrism* __restrict__ lp, int ns, const double* __restrict__ sxyz,
                long long chunk_len, int method, double* __restrict__ partial) {
  // method 0: every pair closed form in double; 1: mixed / float split
  const int s = blockIdx.x * F64_TS + threadIdx.x;
  if (s >= ns) return;
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  float sxh, sxl, syh, syl, szh, szl;
  split2(xs / LIST_L0, &sxh, &sxl);
  split2(ys / LIST_L0, &syh, &syl);
  split2(zs / LIST_L0, &szh, &szl);
  const long long q0 = (long long)blockIdx.y * chunk_len;
  const long long q1 = min(np, q0 + chunk_len);
  double near = 0.0;
  Kahan far;
  for (long long q = q0; q < q1; q++) {
    const double r = rho[q];
    if (r == 0.0) continue;
    bool closed = (method == 0);
    float X = 0.f, Y = 0.f, Z = 0.f, R2 = 0.f;
    ListPrism p;
    if (!closed) {
      p = lp[q];
      X = (sxh - p.xh) + (sxl - p.xl);
      Y = (syh - p.yh) + (syl - p.yl);
      Z = (szh - p.zh) + (szl - p.zl);
      R2 = X * X + Y * Y + Z * Z;
      closed = R2 < p.ell2;
    }
    if (closed) {
      const double* g = geom + 6 * q;
      if (F64NEAR || method == 0) {
        near += r * ztm_prism_unit<double>(g[0] - xs, g[1] - xs, g[2] - ys, g[3] - ys,
                                           g[4] - zs, g[5] - zs);
      } else {
        near += r * (double)ztm_prism_unit<float>(
                        (float)(g[0] - xs), (float)(g[1] - xs), (float)(g[2] - ys),
                        (float)(g[3] - ys), (float)(g[4] - zs), (float)(g[5] - zs));
      }
    } else {
      const float X2 = X * X, Y2 = Y * Y, rh = X2 + Y2;
      const float a0 = fmaf(X2, p.fc.cA, Y2 * p.fc.cB);
      const float h1 = fmaf(X2, p.fc.cX1, Y2 * p.fc.cY1);
      const float h0 = fmaf(X2, fmaf(X2, p.fc.cXX, Y2 * p.fc.cXY), Y2 * Y2 * p.fc.cYY);
      far.add(far_pair(p.w, Z, rh, a0, h0, h1, p.fc));
    }
  }
  // far sum is in km^3 * km / km^3 = 1/km units -> metres: * (L0 km^2 -> m)
  partial[(size_t)blockIdx.y * ns + s] = near + LIST_L0 * far.value();
}

// ---------------------------------------------------------------------------
struct FarShape {
  int tiles, chunks, chunk_cols, sc, grid;
  size_t smem;
};

// Launch shapes the autotuner tries: {columns per shared-memory stage, work
// items per resident block}.  The first is the default.
constexpr int FAR_SHAPES[][2] = {{32, 8}, {16, 16}, {16, 8}, {32, 16}, {64, 16}, {64, 8}};

// Launch shape of the far kernel: sc columns per stage, the grid = the blocks
// resident at once, about ipb work items per block (more items: a shorter
// tail when blocks finish unevenly; fewer: less partial-sum traffic).
FarShape far_shape(const MeshConst& k, int ns, int num_sms, const ztm_opts* o, int sc_want = 16,
                   int ipb = 16) {
  FarShape f;
  f.tiles = std::max(1, (ns + FAR_TS - 1) / FAR_TS);
  int sc = std::max(1, (24 * 1024) / (k.nzp * 4));
  sc = std::min(sc, 64);
  if (sc_want > 0) sc = std::max(1, std::min(sc, sc_want));
  f.sc = sc;
  f.smem = 128 + 2 * (size_t)sc * k.nzp * 4;
  // stages above the default 48 KB need the opt-in (very deep meshes)
  if (f.smem > 48 * 1024 &&
      (cudaFuncSetAttribute(far_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)f.smem) != cudaSuccess ||
       cudaFuncSetAttribute(far_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)f.smem) != cudaSuccess))
    cudaGetLastError();
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, far_kernel<false>, FAR_TS, f.smem) !=
          cudaSuccess ||
      occ < 1) {
    cudaGetLastError();
    occ = 1;
  }
  const long long resident = (long long)occ * std::max(num_sms, 1);
  long long chunks = (ipb * resident + f.tiles - 1) / f.tiles;
  if (o && o->chunk > 0) chunks = (k.ncols + o->chunk - 1) / o->chunk;
  chunks = std::max(1LL, std::min(chunks, (long long)std::max(1, k.ncols / sc)));
  int cc = (int)((k.ncols + chunks - 1) / chunks);
  cc = ((cc + sc - 1) / sc) * sc;
  f.chunk_cols = cc;
  f.chunks = (k.ncols + cc - 1) / cc;
  f.grid = (int)std::min(resident, (long long)f.tiles * f.chunks);
  return f;
}

std::vector<long long> tune_key(const MeshConst& k, int ns) {
  return {1, k.nx, k.ny, k.nz, ns};
}

long long f64_chunks(long long np, int tiles, int num_sms, long long* len) {
  long long want = std::max(1LL, (long long)(8 * std::max(num_sms, 1)) / tiles);
  long long maxc = std::max(1LL, np / 256);
  long long ch = std::min(std::min(want, maxc), 65535LL);
  long long l = (np + ch - 1) / ch;
  l = ((l + 255) / 256) * 256;
  *len = l;
  return (np + l - 1) / l;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers shared with other translation units
MeshConst make_mesh_const(const MeshDesc& m, double near_q) {
  MeshConst k;
  k.nx = m.nx; k.ny = m.ny; k.nz = m.nz;
  k.nzp = (m.nz + 7) & ~7;
  k.ncols = m.nx * m.ny;
  near_widths(m.dx, m.dy, m.dz, near_q, &k.wx, &k.wy, &k.wl);
  k.L0 = std::max(m.dx, std::max(m.dy, m.dz));
  k.dxn = (float)(m.dx / k.L0);
  k.dyn = (float)(m.dy / k.L0);
  k.dzn = (float)(m.dz / k.L0);
  k.fc = far_coef(m.dx / k.L0, m.dy / k.L0, m.dz / k.L0);
  const double ell = 0.5 * sqrt(m.dx * m.dx + m.dy * m.dy + m.dz * m.dz) / k.L0;
  k.rh_t2 = (float)((48.0 * ell) * (48.0 * ell));
  k.dxm = m.dx;
  k.dym = m.dy;
  k.dzm = m.dz;
  const double R = near_q * 0.5 * sqrt(m.dx * m.dx + m.dy * m.dy + m.dz * m.dz);
  k.R2 = R * R;
  k.nslots = (2 * k.wx + 1) * (2 * k.wy + 1);
  return k;
}

void launch_mesh_station_prep(ztm_ctx* c, const MeshDesc& m, double L0, int ns,
                              const double* sxyz, float4* sf, int4* si) {
  if (ns <= 0) return;
  station_prep_kernel<<<(ns + 127) / 128, 128, 0, c->stream>>>(m, L0, ns, sxyz, sf, si);
  c->launches++;
}

void launch_mesh_transpose(ztm_ctx* c, const MeshConst& k, int nmodels, const double* rho,
                           float* rhoT) {
  long long total = (long long)nmodels * k.ncols * k.nzp;
  int blocks = (int)std::min<long long>((total + 255) / 256, 32LL * std::max(c->num_sms, 1));
  transpose_kernel<<<std::max(blocks, 1), 256, 0, c->stream>>>(k, nmodels, rho, rhoT);
  c->launches++;
}

void launch_mesh_near_iv(ztm_ctx* c, const MeshConst& k, const MeshDesc& m, int ns,
                         const int4* si, const double* sxyz, short2* iv, int2* lr) {
  if (ns <= 0) return;
  near_iv_kernel<<<ns, NEAR_IV_TS, 0, c->stream>>>(k, m, ns, si, sxyz, iv, lr);
  c->launches++;
}

size_t ztm_prism_ws(const MeshDesc& m, int ns, int precision, int num_sms, const ztm_opts* o) {
  if (precision == ZTM_PREC_FP64) {
    const long long nv = (long long)(m.nx + 1) * (m.ny + 1) * (m.nz + 1);
    long long len;
    int tiles = std::max(1, (ns + F64_TS - 1) / F64_TS);
    long long ch = f64_chunks(nv, tiles, num_sms, &len);
    return WsCarver::need((size_t)ch * ns * 8) + WsCarver::need((size_t)nv * 8);
  }
  double nq = (o && o->near_q > 0) ? o->near_q : ZTM_MESH_NEAR_Q;
  MeshConst k = make_mesh_const(m, nq);
  int chunks = 0;
  for (const auto& sh : FAR_SHAPES)
    chunks = std::max(chunks, far_shape(k, ns, num_sms, o, sh[0], sh[1]).chunks);
  return WsCarver::need(sizeof(int)) + WsCarver::need((size_t)k.ncols * k.nzp * 4) +
         WsCarver::need((size_t)ns * 16) * 2 + WsCarver::need((size_t)ns * 4) +
         ztm_station_order_ws(ns, m.nx, m.ny) +
         WsCarver::need((size_t)ns * 8) + WsCarver::need((size_t)chunks * ns * 8) +
         WsCarver::need((size_t)ns * k.nslots * 4) + WsCarver::need((size_t)ns * 8);
}

int ztm_launch_prism(ztm_ctx* c, const MeshDesc& m, const double* d_rho, int ns,
                     const double* d_sxyz, double* d_gz, double G, int precision,
                     const ztm_opts* o, WsCarver& wc) {
  const double G5 = G * 1.0e5;
  if (precision == ZTM_PREC_FP64) {
    const long long nv = (long long)(m.nx + 1) * (m.ny + 1) * (m.nz + 1);
    if (nv > (1LL << 31) - 1) return ztm_fail(c, ZTM_ERR_RANGE, "mesh has more than 2^31-1 vertices");
    long long len;
    int tiles = std::max(1, (ns + F64_TS - 1) / F64_TS);
    long long ch = f64_chunks(nv, tiles, c->num_sms, &len);
    double* partial = wc.take<double>((size_t)ch * ns);
    double* D = wc.take<double>((size_t)nv);
    vertex_weight_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, c->stream>>>(m, d_rho, D);
    {
      ZtmProf prof_(c, "prism_f64");
      mesh_f64_kernel<<<dim3(tiles, (unsigned)ch), F64_TS, 0, c->stream>>>(m, ns, d_sxyz, D, len,
                                                                           partial);
    }
    finalize_kernel<<<(ns + 255) / 256, 256, 0, c->stream>>>(ns, (int)ch, partial, 1.0, nullptr,
                                                             G5, d_gz);
    c->launches += 3;
    return ztm_after_launch(c, "prism FP64 kernels");
  }
  const double nq = (o && o->near_q > 0) ? o->near_q : ZTM_MESH_NEAR_Q;
  MeshConst k = make_mesh_const(m, nq);
  if (m.nz > 32767) return ztm_fail(c, ZTM_ERR_RANGE, "mixed prism forward supports nz <= 32767");
  {  // two one-column stages of the far kernel must fit in shared memory
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    const long long nzp = (m.nz + 7) & ~7;
    if (optin > 0 && 128 + 8 * nzp > optin)
      return ztm_fail(c, ZTM_ERR_RANGE,
                      "mixed prism forward: nz too large for two one-column stages in shared memory");
  }
  int shape = 0;
  auto it = c->tuned.find(tune_key(k, ns));
  if (it != c->tuned.end()) shape = (int)it->second[0];
  int* counter = wc.take<int>(1);
  float* rhoT = wc.take<float>((size_t)k.ncols * k.nzp);
  float4* sf = wc.take<float4>(ns);
  int4* si = wc.take<int4>(ns);
  double* near = wc.take<double>(ns);
  int max_chunks = 0;
  for (const auto& sh : FAR_SHAPES)
    max_chunks = std::max(max_chunks, far_shape(k, ns, c->num_sms, o, sh[0], sh[1]).chunks);
  double* partial = wc.take<double>((size_t)max_chunks * ns);
  short2* iv = wc.take<short2>((size_t)ns * k.nslots);
  int2* lr = wc.take<int2>(ns);
  launch_mesh_transpose(c, k, 1, d_rho, rhoT);
  launch_mesh_station_prep(c, m, k.L0, ns, d_sxyz, sf, si);
  int* perm = wc.take<int>(ns);
  if (int rc = ztm_station_order(c, c->stream, ns, reinterpret_cast<const int*>(si), 4, m.nx, m.ny,
                                 perm, wc))
    return rc;
  launch_mesh_near_iv(c, k, m, ns, si, d_sxyz, iv, lr);
  FarArgs a;
  a.k = k; a.ns = ns; a.sf = sf; a.si = si; a.iv = iv; a.rhoT = rhoT; a.partial = partial;
  a.perm = perm;
  a.err = c->d_err;
  a.counter = counter;
  a.n_near = (ns + FAR_NEAR_ST - 1) / FAR_NEAR_ST;
  a.near_f64 = precision == ZTM_PREC_MIXED;
  a.m = m;
  a.sxyz = d_sxyz;
  a.rho = d_rho;
  a.lr = lr;
  a.near = near;
  a.poll_limit = c->stage_wait_limit;
  a.forms = c->d_forms;
  auto launch_far = [&](const FarShape& t) {
    a.tiles = t.tiles;
    a.chunks = t.chunks;
    a.chunk_cols = t.chunk_cols;
    a.sc = t.sc;
    cudaMemsetAsync(counter, 0, sizeof(int), c->stream);
    if (c->count_forms && c->d_forms)
      far_kernel<true><<<t.grid, FAR_TS, t.smem, c->stream>>>(a);
    else
      far_kernel<false><<<t.grid, FAR_TS, t.smem, c->stream>>>(a);
    c->launches++;
  };
  if (o && (o->flags & ZTM_FLAG_AUTOTUNE) && !(o->chunk > 0) && it == c->tuned.end()) {
    // time each candidate once (after one untimed launch) and keep the fastest
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    const int nshapes = (int)(sizeof(FAR_SHAPES) / sizeof(FAR_SHAPES[0]));
    for (int q = 0; q < nshapes; q++) {
      FarShape t = far_shape(k, ns, c->num_sms, o, FAR_SHAPES[q][0], FAR_SHAPES[q][1]);
      launch_far(t);
      cudaEventRecord(e0, c->stream);
      launch_far(t);
      cudaEventRecord(e1, c->stream);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) ==
                                                         cudaSuccess && ms < best) {
        best = ms;
        shape = q;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->tuned[tune_key(k, ns)] = {shape};
  }
  FarShape f = far_shape(k, ns, c->num_sms, o, FAR_SHAPES[shape][0], FAR_SHAPES[shape][1]);
  // near regions (FP64 pipe) and far fields (FMA pipe) in one persistent grid
  {
    ZtmProf prof_(c, "prism_far");
    launch_far(f);
  }
  const double far_scale = k.L0 * (double)k.dxn * k.dyn * k.dzn;
  finalize_kernel<<<(ns + 255) / 256, 256, 0, c->stream>>>(ns, f.chunks, partial, far_scale, near,
                                                           G5, d_gz);
  c->launches++;
  return ztm_after_launch(c, "prism mixed kernels");
}

size_t ztm_prism_list_ws(long long np, int ns, int precision, int num_sms) {
  int tiles = std::max(1, (ns + F64_TS - 1) / F64_TS);
  long long len;
  long long ch = f64_chunks(std::max(np, 1LL), tiles, num_sms, &len);
  size_t w = WsCarver::need((size_t)ch * ns * 8);
  if (precision != ZTM_PREC_FP64) w += WsCarver::need((size_t)np * sizeof(ListPrism));
  return w;
}

int ztm_launch_prism_list(ztm_ctx* c, long long np, const double* d_geom, const double* d_rho,
                          int ns, const double* d_sxyz, double* d_gz, double G, int precision,
                          double near_q, WsCarver& wc) {
  const double G5 = G * 1.0e5;
  int tiles = std::max(1, (ns + F64_TS - 1) / F64_TS);
  long long len;
  long long ch = f64_chunks(std::max(np, 1LL), tiles, c->num_sms, &len);
  double* partial = wc.take<double>((size_t)ch * ns);
  ListPrism* lp = nullptr;
  if (precision != ZTM_PREC_FP64 && np > 0) {
    lp = wc.take<ListPrism>(np);
    list_prep_kernel<<<(unsigned)((np + 255) / 256), 256, 0, c->stream>>>(np, d_geom, d_rho,
                                                                          near_q, lp);
    c->launches++;
  }
  if (np > 0) {
    dim3 grid(tiles, (unsigned)ch);
    int method = precision == ZTM_PREC_FP64 ? 0 : 1;
    if (precision == ZTM_PREC_FP32)
      {
        ZtmProf prof_(c, "prism_list");
        list_kernel<false><<<grid, F64_TS, 0, c->stream>>>(np, d_geom, d_rho, lp, ns, d_sxyz, len,
                                                           method, partial);
      }
    else
      {
        ZtmProf prof_(c, "prism_list");
        list_kernel<true><<<grid, F64_TS, 0, c->stream>>>(np, d_geom, d_rho, lp, ns, d_sxyz, len,
                                                          method, partial);
      }
    c->launches++;
  } else {
    ch = 0;
  }
  finalize_kernel<<<(ns + 255) / 256, 256, 0, c->stream>>>(ns, (int)ch, partial, 1.0, nullptr, G5,
                                                           d_gz);
  c->launches++;
  return ztm_after_launch(c, "prism list kernels");
}
