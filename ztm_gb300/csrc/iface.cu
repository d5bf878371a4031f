// iface.cu - interface (prism-column) model: forward, adjoint and misfit.
//
// Column c = (ix, iy) spans its cell horizontally and z in [z_base, -depth[c]]
// with density rho[c].  gz(s) = G*1e5 * sum_c rho[c] * U(s, c), U the prism
// integral of (z_s - z)/r^3.  The adjoint gives
//   g_rho[c]   = G*1e5 * sum_s r[s] * U(s, c)
//   g_depth[c] = -G*1e5 * rho[c] * sum_s r[s] * F(s, c),
// F the integral of (z_s - z_top)/r^3 over the column's top face (the
// analytic derivative of U with respect to the top, 4-corner atan sum).
// This is the Moho-interface parameterisation of the reference's density
// builder (TFM.cpp:85-88), where a column's density contrast switches at the
// rendered Moho depth; the reference differentiates it only by finite
// differences of full forward runs (TFM.cpp:124-135).
//
// Mixed method.  Far columns: the vertical integral is exact,
//   1/r_top - 1/r_base = thick (u_t + u_b) / (r_t r_b (r_t + r_b)),
// written without cancellation, and the horizontal integral over the cell
// is the 4th-order Taylor expansion of 1/r in (X, Y):
//   C(u) = (Q2 + Q0 r^2)/r^5 + (P4 + P2 r^2 + P0 r^4)/r^9,
// with Q2 = (dx^2 X^2 + dy^2 Y^2)/8, Q0 = -(dx^2 + dy^2)/24,
//      P4 = 7/128 (dx^4 X^4 + dy^4 Y^4) + 35/192 dx^2 dy^2 X^2 Y^2,
//      P2 = -3/64 (dx^4 X^2 + dy^4 Y^2) - 5/192 dx^2 dy^2 (X^2 + Y^2),
//      P0 = 3/640 (dx^4 + dy^4) + 1/192 dx^2 dy^2,
// so U ~ dx dy [1/r_t - 1/r_b + C(u_t) - C(u_b)].  The face term is the 2-D
// form of the prism far-field expansion (dz = 0).  All in float with Kahan
// sums.  Near columns (within near_q horizontal half-diagonals of the
// station's home column) use the closed forms in double.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "prism_common.cuh"
#include "ztm_internal.cuh"

namespace {

constexpr int IF_TS = 128;
constexpr int IF_TILE = 256;
constexpr int IF_NEAR_WPB = 4;
// forward blocks per SM to aim for (waves x residency): the Moho forward
// took 1.75 ms at 8 (under one wave), 1.6 at 24, 1.55 at 48
constexpr int IF_FWD_PER_SM = 48;
constexpr int IF_SUB = 32;       // columns per second-order test in the forward
constexpr float IF_FAR = 1.0e6f; // -index of a padding column (far away)
// the forward's tile load: each warp loads whole blocks of IF_SUB columns
static_assert(IF_SUB == 32 && IF_TILE % IF_TS == 0 && IF_TS % 32 == 0, "tile load layout");

struct IConst {
  int nx, ny, ncols, w;  // w: near window half width (columns)
  int words;             // 32-bit mask words per station ((2w+1)^2 bits)
  double near_h;         // near_q * horizontal half diagonal (m)
  float dxn, dyn;
  double L0;
  float Q0, P0;
  float q2x, q2y;        // Q2 = q2x X^2 + q2y Y^2
  float p4x, p4y, p4xy;  // P4
  float p2x, p2y;        // P2 = p2x X^2 + p2y Y^2
  FarCoef face;          // 2-D face expansion
  float rt2_t2;          // squared distance to the column top (units of L0)
                         // beyond which the 4th-order terms are dropped
};

IConst make_iconst(const IMeshDesc& m, double near_q) {
  IConst k;
  k.nx = m.nx;
  k.ny = m.ny;
  k.ncols = m.nx * m.ny;
  k.L0 = std::max(m.dx, m.dy);
  double dx = m.dx / k.L0, dy = m.dy / k.L0;
  k.dxn = (float)dx;
  k.dyn = (float)dy;
  double x2 = dx * dx, y2 = dy * dy, x4 = x2 * x2, y4 = y2 * y2;
  k.q2x = (float)(x2 / 8);
  k.q2y = (float)(y2 / 8);
  k.Q0 = (float)(-(x2 + y2) / 24);
  k.p4x = (float)(7.0 / 128 * x4);
  k.p4y = (float)(7.0 / 128 * y4);
  k.p4xy = (float)(35.0 / 192 * x2 * y2);
  k.p2x = (float)(-3.0 / 64 * x4 - 5.0 / 192 * x2 * y2);
  k.p2y = (float)(-3.0 / 64 * y4 - 5.0 / 192 * x2 * y2);
  k.P0 = (float)(3.0 / 640 * (x4 + y4) + 1.0 / 192 * x2 * y2);
  k.face = far_coef(dx, dy, 0.0);
  double ellh = 0.5 * sqrt(m.dx * m.dx + m.dy * m.dy);
  int w = (int)ceil(near_q * ellh / std::min(m.dx, m.dy) - 0.5);
  k.w = std::max(w, 0);
  k.words = ((2 * k.w + 1) * (2 * k.w + 1) + 31) / 32;
  // vertically the column's top face is what the station sees first; its
  // face term converges more slowly than the column's, so keep columns in
  // double until the station is twice as far above the top
  k.near_h = 2.0 * near_q * ellh;
  // 96 horizontal half diagonals: the dropped 4th-order horizontal terms of
  // the column and of its top face are below 1e-8 of the pair's monopole
  k.rt2_t2 = (float)((96.0 * ellh / k.L0) * (96.0 * ellh / k.L0));
  return k;
}

struct IStation {  // per-station float data
  float ex, ey, zs, r;
};

__global__ void iface_station_prep(IMeshDesc m, double L0, int ns, const double* __restrict__ sxyz,
                                   const double* __restrict__ res, IStation* __restrict__ sf,
                                   int2* __restrict__ si) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  const double lim = 1.0e9;
  int ix = (int)fmin(fmax(floor((xs - m.x0) / m.dx), -lim), lim);
  int iy = (int)fmin(fmax(floor((ys - m.y0) / m.dy), -lim), lim);
  IStation f;
  f.ex = (float)(((xs - m.x0) - (ix + 0.5) * m.dx) / L0);
  f.ey = (float)(((ys - m.y0) - (iy + 0.5) * m.dy) / L0);
  f.zs = (float)(zs / L0);
  f.r = res ? (float)res[s] : 0.f;
  sf[s] = f;
  si[s] = make_int2(ix, iy);
}

// per column: (rho, depth/L0, thickness/L0, 0)
// Per-column float data: (weight, top depth, thickness) in units of L0.  The
// weight is rho, or rho * vdep[c] for the depth directional derivative.
__global__ void iface_col_prep(IMeshDesc m, double L0, const double* __restrict__ depth,
                               const double* __restrict__ rho, const double* __restrict__ vdep,
                               float4* __restrict__ cf) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= (long long)m.nx * m.ny) return;
  double d = depth[c];
  double thick = (-d - m.zb) / L0;
  const double w = vdep ? rho[c] * vdep[c] : rho[c];
  cf[c] = make_float4((float)w, (float)(d / L0), (float)thick, 0.f);
}

// Near columns of a station: inside the (2w+1)^2 window around its home
// column (clamped to the mesh) AND with the station less than near_h
// (2 near_q half-diagonals) above the column's top.  Outside the window the
// horizontal distance alone is >= near_q half-diagonals; inside it, a station
// that high above the top is at least as far from every point of the column.
// The window slot of (ix, iy):
__device__ __forceinline__ bool window_slot(int ixs, int iys, int ix, int iy, const IConst& k,
                                            int* slot) {
  const int cx = clampi(ixs, 0, k.nx - 1), cy = clampi(iys, 0, k.ny - 1);
  if (abs(ix - cx) > k.w || abs(iy - cy) > k.w) return false;
  const int x0 = max(0, cx - k.w), x1 = min(k.nx - 1, cx + k.w), y0 = max(0, cy - k.w);
  *slot = (ix - x0) + (x1 - x0 + 1) * (iy - y0);
  return true;
}

// The near bit of (station, column), from the mask the mask kernel wrote.
__device__ __forceinline__ bool is_near(const uint32_t* __restrict__ mask, int s, int ixs, int iys,
                                        int ix, int iy, const IConst& k) {
  int slot;
  if (!window_slot(ixs, iys, ix, iy, k, &slot)) return false;
  return (__ldg(mask + (size_t)s * k.words + (slot >> 5)) >> (slot & 31)) & 1u;
}

// The near bit of window slot `slot` of station s.
__device__ __forceinline__ bool near_bit(const uint32_t* __restrict__ mask, int s, int slot,
                                         const IConst& k) {
  return (__ldg(mask + (size_t)s * k.words + (slot >> 5)) >> (slot & 31)) & 1u;
}

// One warp per station: the near bit of every window column, in double.
__global__ void iface_near_mask(IConst k, int ns, const double* __restrict__ sxyz,
                                const int2* __restrict__ si, const double* __restrict__ depth,
                                uint32_t* __restrict__ mask, int* __restrict__ anynear) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * 4 + warp;
  if (s >= ns) return;
  const int2 h = si[s];
  const int cx = clampi(h.x, 0, k.nx - 1), cy = clampi(h.y, 0, k.ny - 1);
  const int x0 = max(0, cx - k.w), x1 = min(k.nx - 1, cx + k.w);
  const int y0 = max(0, cy - k.w), y1 = min(k.ny - 1, cy + k.w);
  const int wx = x1 - x0 + 1, n = wx * (y1 - y0 + 1);
  const double zs = sxyz[3 * s + 2];
  uint32_t any = 0u;
  for (int wd = 0; wd < k.words; wd++) {
    const int q = wd * 32 + lane;
    bool nb = false;
    if (q < n) {
      const int ix = x0 + q % wx, iy = y0 + q / wx;
      nb = zs + depth[ix + (long long)k.nx * iy] < k.near_h;  // zs - z_top < near_h
    }
    const uint32_t bits = __ballot_sync(0xffffffffu, nb);
    if (lane == 0) mask[(size_t)s * k.words + wd] = bits;
    any |= bits;
  }
  if (lane == 0) anynear[s] = any != 0u;  // the station has a near column
}

// The unit face integral of the far expansion for two pairs, given 1/r of
// the column top.  T2: second order only (pairs beyond rt2_t2).
template <bool T2>
__device__ __forceinline__ float2 face_unit_far2(float2 X2, float2 Y2, float2 ut, float2 rinv,
                                                 const FarCoef& f) {
  const float2 Z2 = __fmul2_rn(ut, ut);
  const float2 ri2 = __fmul2_rn(rinv, rinv), ri4 = __fmul2_rn(ri2, ri2);
  const float2 a0 = __ffma2_rn(X2, make_float2(f.cA, f.cA), __fmul2_rn(Y2, make_float2(f.cB, f.cB)));
  const float2 n2 = __ffma2_rn(make_float2(f.a1, f.a1), Z2, a0);
  float2 t;
  if (T2) {
    t = __fmul2_rn(n2, ri4);
  } else {
    const float2 h1 = __ffma2_rn(X2, make_float2(f.cX1, f.cX1), __fmul2_rn(Y2, make_float2(f.cY1, f.cY1)));
    const float2 h0 = __ffma2_rn(
        X2, __ffma2_rn(X2, make_float2(f.cXX, f.cXX), __fmul2_rn(Y2, make_float2(f.cXY, f.cXY))),
        __fmul2_rn(__fmul2_rn(Y2, Y2), make_float2(f.cYY, f.cYY)));
    const float2 H = __ffma2_rn(__ffma2_rn(make_float2(f.h2, f.h2), Z2, h1), Z2, h0);
    t = __fmul2_rn(__ffma2_rn(H, ri4, n2), ri4);
  }
  const float2 base = __fmul2_rn(__fmul2_rn(ut, rinv), ri2);
  return __ffma2_rn(base, t, base);
}

// Unit column integral (normalised, without dx dy) for two far pairs on the
// packed FP32 path: the exact vertical integral of the column axis plus the
// horizontal correction at its top and bottom, to 4th order, or to 2nd order
// when T2 (pairs beyond rt2_t2).  rt2 = ut^2 + rh.  The SFU operations stay
// scalar.  Also hands back 1/r of the column top.
template <bool T2>
__device__ __forceinline__ float2 col_unit2(float2 X2, float2 Y2, float2 rh, float2 ut,
                                            float2 rt2, float2 th, const IConst& k,
                                            float2* it_out) {
  const float2 Q2 = __ffma2_rn(make_float2(k.q2x, k.q2x), X2, __fmul2_rn(make_float2(k.q2y, k.q2y), Y2));
  const float2 ub = __fadd2_rn(ut, th);
  const float2 rb2 = __ffma2_rn(ub, ub, rh);
  const float2 it = make_float2(rsqrt_ftz(rt2.x), rsqrt_ftz(rt2.y));
  const float2 ib = make_float2(rsqrt_ftz(rb2.x), rsqrt_ftz(rb2.y));
  *it_out = it;
  const float2 itb = __fmul2_rn(it, ib);
  const float2 num = __fmul2_rn(__fmul2_rn(th, __fadd2_rn(ut, ub)), __fmul2_rn(itb, itb));
  const float2 den = __fadd2_rn(it, ib);
  const float2 L = make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
  // the corrections it^5 (Q0 rt^2 + Q2) + it^9 (P0 rt^4 + P2 rt^2 + P4) at the
  // top (and the same at the bottom), with rt^2 it^2 = 1 folded in:
  //   it^3 (Q0 + it^2 ((Q2 + P0) + it^2 (P2 + it^2 P4)))
  const float2 Q0 = make_float2(k.Q0, k.Q0);
  const float2 it2 = __fmul2_rn(it, it), ib2 = __fmul2_rn(ib, ib);
  const float2 it3 = __fmul2_rn(it2, it), ib3 = __fmul2_rn(ib2, ib);
  float2 ct, cb;
  if (T2) {
    ct = __fmul2_rn(it3, __ffma2_rn(it2, Q2, Q0));
    cb = __fmul2_rn(ib3, __ffma2_rn(ib2, Q2, Q0));
  } else {
    const float2 P4 = __ffma2_rn(__fmul2_rn(make_float2(k.p4x, k.p4x), X2), X2,
                                 __ffma2_rn(__fmul2_rn(make_float2(k.p4y, k.p4y), Y2), Y2,
                                            __fmul2_rn(__fmul2_rn(make_float2(k.p4xy, k.p4xy), X2), Y2)));
    const float2 P2 = __ffma2_rn(make_float2(k.p2x, k.p2x), X2, __fmul2_rn(make_float2(k.p2y, k.p2y), Y2));
    const float2 QP = __fadd2_rn(Q2, make_float2(k.P0, k.P0));
    ct = __fmul2_rn(it3, __ffma2_rn(it2, __ffma2_rn(it2, __ffma2_rn(it2, P4, P2), QP), Q0));
    cb = __fmul2_rn(ib3, __ffma2_rn(ib2, __ffma2_rn(ib2, __ffma2_rn(ib2, P4, P2), QP), Q0));
  }
  return __fadd2_rn(L, __fadd2_rn(ct, make_float2(-cb.x, -cb.y)));
}

// ---- forward, far (thread per station) ------------------------------------
// Columns stream through shared memory in tiles, with their indices as
// negated floats (exact) so that the offsets need no integer work.  The
// near-window test runs only in warps where some station has a near column
// (anynear, from the mask kernel): for stations well above the interface it
// never runs.
// FACE: the top-face integral instead of the column integral (the depth
// directional derivative, with the columns weighted by rho * direction).
template <bool FACE>
__global__ void __launch_bounds__(IF_TS, 8)
    iface_far_fwd(IConst k, int ns, const IStation* __restrict__ sf, const int2* __restrict__ si,
                  const float4* __restrict__ cf, const uint32_t* __restrict__ mask,
                  const int* __restrict__ anynear, const int* __restrict__ perm, int chunk_len,
                  double* __restrict__ partial) {
  // the tile's columns, one array per field so that a column pair is one
  // 8-byte load per field (weight, top depth, thickness, -ix, -iy)
  __shared__ __align__(8) float s_w[IF_TILE + 2];
  __shared__ __align__(8) float s_top[IF_TILE + 2];
  __shared__ __align__(8) float s_th[IF_TILE + 2];
  __shared__ __align__(8) float s_nx[IF_TILE + 2];  // -ix of the tile's columns
  __shared__ __align__(8) float s_ny[IF_TILE + 2];  // -iy
  __shared__ float s_tmin[IF_TILE / IF_SUB];         // shallowest top per column block
  const int slot = blockIdx.x * IF_TS + threadIdx.x;  // stations in Z order
  const bool active = slot < ns;
  const int s = active ? perm[slot] : 0;
  IStation st = {0.f, 0.f, 0.f, 0.f};
  int2 hi = make_int2(0, 0);
  bool mine_near = false;
  if (active) {
    st = sf[s];
    hi = si[s];
    mine_near = anynear[s] != 0;
  }
  const bool warp_near = __any_sync(0xffffffffu, mine_near);
  const int c0 = blockIdx.y * chunk_len, c1 = min(k.ncols, c0 + chunk_len);
  // this station's near window (clamped), for the per-column test
  const int wcx = clampi(hi.x, 0, k.nx - 1), wcy = clampi(hi.y, 0, k.ny - 1);
  const int wx0 = active ? max(0, wcx - k.w) : 1, wx1 = active ? min(k.nx - 1, wcx + k.w) : 0;
  const int wy0 = max(0, wcy - k.w), wy1 = min(k.ny - 1, wcy + k.w);
  const int wbw = wx1 - wx0 + 1;
  const float2 hx2 = make_float2((float)hi.x, (float)hi.x), hy2 = make_float2((float)hi.y, (float)hi.y);
  const float2 dxn2 = make_float2(k.dxn, k.dxn), dyn2 = make_float2(k.dyn, k.dyn);
  const float2 ex2 = make_float2(st.ex, st.ex), ey2 = make_float2(st.ey, st.ey);
  const float2 zs2 = make_float2(st.zs, st.zs);
  Kahan acc;
  for (int t0 = c0; t0 < c1; t0 += IF_TILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < IF_TILE + 2; q += IF_TS) {
      const int c = t0 + q;
      const bool ok = c < c1;
      const float4 cq = ok ? cf[c] : make_float4(0.f, 0.f, 0.f, 0.f);
      s_w[q] = cq.x;
      s_top[q] = cq.y;
      s_th[q] = cq.z;
      // a padding column has zero weight and lies far away: its terms are
      // finite and add zero
      s_nx[q] = ok ? -(float)(c % k.nx) : IF_FAR;
      s_ny[q] = ok ? -(float)(c / k.nx) : IF_FAR;
      // the shallowest top of each block of IF_SUB columns (a warp loads one)
      if (q < IF_TILE) {
        float t = ok ? cq.y : 3.0e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = fminf(t, __shfl_xor_sync(0xffffffffu, t, o));
        if ((q & (IF_SUB - 1)) == 0) s_tmin[q / IF_SUB] = t;
      }
    }
    __syncthreads();
    if (!active) continue;
    const int cnt = min(IF_TILE, c1 - t0);
    for (int q0 = 0; q0 < cnt; q0 += IF_SUB) {
      const int qe = min(cnt, q0 + IF_SUB);
      // second order for the whole block when every station of the warp is
      // far enough from every column of it: a lower bound of the squared
      // distance to a column top from the block's column and row ranges
      const int ca = t0 + q0, cb = t0 + qe - 1;
      const int ya = ca / k.nx, yb = cb / k.nx;
      const int xa = ya == yb ? ca % k.nx : 0, xb = ya == yb ? cb % k.nx : k.nx - 1;
      auto gap = [](float lo, float hi) {  // min |v| for v between lo and hi
        return (lo <= 0.f && hi >= 0.f) ? 0.f : fminf(fabsf(lo), fabsf(hi));
      };
      const float gx = gap(fmaf((float)(hi.x - xb), k.dxn, st.ex), fmaf((float)(hi.x - xa), k.dxn, st.ex));
      const float gy = gap(fmaf((float)(hi.y - yb), k.dyn, st.ey), fmaf((float)(hi.y - ya), k.dyn, st.ey));
      const float gz = fmaxf(0.f, st.zs + s_tmin[q0 / IF_SUB]);
      const bool t2 = __all_sync(__activemask(), fmaf(gz, gz, fmaf(gx, gx, gy * gy)) >= k.rt2_t2);
      auto run = [&](auto t2c) {
        constexpr bool T2 = decltype(t2c)::value;
        float2 g = make_float2(0.f, 0.f);  // plain sums over IF_SUB columns, Kahan across
#pragma unroll 4
        for (int q = q0; q < qe; q += 2) {
          // columns q and q+1 (past the end of the tile: a padding column)
          const float2 nx2 = *reinterpret_cast<const float2*>(s_nx + q);
          const float2 ny2 = *reinterpret_cast<const float2*>(s_ny + q);
          const float2 X = __ffma2_rn(__fadd2_rn(hx2, nx2), dxn2, ex2);
          const float2 Y = __ffma2_rn(__fadd2_rn(hy2, ny2), dyn2, ey2);
          const float2 X2 = __fmul2_rn(X, X), Y2 = __fmul2_rn(Y, Y), rh = __fadd2_rn(X2, Y2);
          const float2 ut = __fadd2_rn(zs2, *reinterpret_cast<const float2*>(s_top + q));
          const float2 rt2 = __ffma2_rn(ut, ut, rh);
          const float2 th = *reinterpret_cast<const float2*>(s_th + q);
          float2 itop, u;
          if (FACE) {
            itop = make_float2(rsqrt_ftz(rt2.x), rsqrt_ftz(rt2.y));
            u = face_unit_far2<T2>(X2, Y2, ut, itop, k.face);
          } else {
            u = col_unit2<T2>(X2, Y2, rh, ut, rt2, th, k, &itop);
          }
          float2 v = __fmul2_rn(*reinterpret_cast<const float2*>(s_w + q), u);
          if (warp_near) {
            // near columns contribute through the double path: select, which
            // also drops a NaN
            const int ixa = -(int)nx2.x, iya = -(int)ny2.x, ixb = -(int)nx2.y, iyb = -(int)ny2.y;
            if (ixa >= wx0 && ixa <= wx1 && iya >= wy0 && iya <= wy1 &&
                near_bit(mask, s, ixa - wx0 + wbw * (iya - wy0), k))
              v.x = 0.f;
            if (ixb >= wx0 && ixb <= wx1 && iyb >= wy0 && iyb <= wy1 &&
                near_bit(mask, s, ixb - wx0 + wbw * (iyb - wy0), k))
              v.y = 0.f;
          }
          g = __fadd2_rn(g, v);
        }
        acc.add(g.x + g.y);
      };
      if (t2)
        run(std::true_type{});
      else
        run(std::false_type{});
    }
  }
  if (active) partial[(size_t)blockIdx.y * ns + s] = acc.value();
}

// ---- forward, near window in double (warp per station) ---------------------
template <bool FACE>
__global__ void iface_near_fwd(IConst k, IMeshDesc m, int ns, const double* __restrict__ sxyz,
                               const int2* __restrict__ si, const double* __restrict__ depth,
                               const double* __restrict__ rho, const double* __restrict__ vdep,
                               const uint32_t* __restrict__ mask, double* __restrict__ out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * IF_NEAR_WPB + warp;
  if (s >= ns) return;
  const int2 h = si[s];
  const int cx = clampi(h.x, 0, k.nx - 1), cy = clampi(h.y, 0, k.ny - 1);
  const int x0 = max(0, cx - k.w), x1 = min(k.nx - 1, cx + k.w);
  const int y0 = max(0, cy - k.w), y1 = min(k.ny - 1, cy + k.w);
  const int wx = x1 - x0 + 1, n = wx * (y1 - y0 + 1);
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  double acc = 0.0;
  for (int q = lane; q < n; q += 32) {
    if (!((mask[(size_t)s * k.words + (q >> 5)] >> (q & 31)) & 1u)) continue;
    const int ix = x0 + q % wx, iy = y0 + q / wx;
    const long long c = ix + (long long)m.nx * iy;
    const double r = FACE ? rho[c] * vdep[c] : rho[c];
    if (r == 0.0) continue;
    const double xa = (m.x0 + ix * m.dx) - xs, xb = (m.x0 + (ix + 1) * m.dx) - xs;
    const double ya = (m.y0 + iy * m.dy) - ys, yb = (m.y0 + (iy + 1) * m.dy) - ys;
    if (FACE)
      acc += r * ztm_face_unit(xa, xb, ya, yb, zs + depth[c]);  // zs - z_top
    else
      acc += r * ztm_prism_unit<double>(xa, xb, ya, yb, m.zb - zs, -depth[c] - zs);
  }
  acc = warp_sum_d(acc);
  if (lane == 0) out[s] = acc;
}

__global__ void iface_finalize(int ns, int nchunks, const double* __restrict__ partial,
                               double far_scale, const double* __restrict__ near, double G5,
                               double* __restrict__ gz) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  double f = 0.0;
  for (int c = 0; c < nchunks; c++) f += partial[(size_t)c * ns + s];
  double g = far_scale * f;
  if (near) g += near[s];
  gz[s] = G5 * g;
}

// ---- forward, plain double --------------------------------------------------
template <bool FACE>
__global__ void __launch_bounds__(64)
    iface_f64_fwd(IMeshDesc m, int ns, const double* __restrict__ sxyz,
                  const double* __restrict__ depth, const double* __restrict__ rho,
                  const double* __restrict__ vdep, int chunk_len, double* __restrict__ partial) {
  const int s = blockIdx.x * 64 + threadIdx.x;
  if (s >= ns) return;
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  const int nc = m.nx * m.ny;
  const int c0 = blockIdx.y * chunk_len, c1 = min(nc, c0 + chunk_len);
  double acc = 0.0;
  for (int c = c0; c < c1; c++) {
    const double r = FACE ? rho[c] * vdep[c] : rho[c];
    if (r == 0.0) continue;
    const int ix = c % m.nx, iy = c / m.nx;
    const double xa = (m.x0 + ix * m.dx) - xs, xb = (m.x0 + (ix + 1) * m.dx) - xs;
    const double ya = (m.y0 + iy * m.dy) - ys, yb = (m.y0 + (iy + 1) * m.dy) - ys;
    if (FACE)
      acc += r * ztm_face_unit(xa, xb, ya, yb, zs + depth[c]);  // zs - z_top
    else
      acc += r * ztm_prism_unit<double>(xa, xb, ya, yb, m.zb - zs, -depth[c] - zs);
  }
  partial[(size_t)blockIdx.y * ns + s] = acc;
}

// ---- adjoint, far (thread per column) --------------------------------------
__global__ void __launch_bounds__(IF_TS, 8)
    iface_far_adj(IConst k, int ns, const IStation* __restrict__ sf, const int2* __restrict__ si,
                  const float4* __restrict__ cf, const uint32_t* __restrict__ mask,
                  const int* __restrict__ anynear, int chunk_len, double* __restrict__ p_rho,
                  double* __restrict__ p_dep) {
  // the tile's stations, one array per field so that a station pair is one
  // 8-byte load per field
  __shared__ __align__(8) float s_ex[IF_TILE + 2];
  __shared__ __align__(8) float s_ey[IF_TILE + 2];
  __shared__ __align__(8) float s_zs[IF_TILE + 2];
  __shared__ __align__(8) float s_r[IF_TILE + 2];
  __shared__ __align__(8) float s_hx[IF_TILE + 2];  // home column indices as floats (exact)
  __shared__ __align__(8) float s_hy[IF_TILE + 2];
  __shared__ int2 s_i[IF_TILE + 2];
  __shared__ int s_nf[IF_TILE + 2];  // the station has a near column
  const int c = blockIdx.x * IF_TS + threadIdx.x;
  const bool active = c < k.ncols;
  const int ix = active ? c % k.nx : 0, iy = active ? c / k.nx : 0;
  const float4 col = active ? cf[c] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float2 cy2 = make_float2(col.y, col.y), cz2 = make_float2(col.z, col.z);
  const float2 nix2 = make_float2(-(float)ix, -(float)ix), niy2 = make_float2(-(float)iy, -(float)iy);
  const float2 dxn2 = make_float2(k.dxn, k.dxn), dyn2 = make_float2(k.dyn, k.dyn);
  // this block's slice of the stations (grid.y)
  const int s0 = blockIdx.y * chunk_len, s1 = min(ns, s0 + chunk_len);
  Kahan ar, ad;
  for (int t0 = s0; t0 < s1; t0 += IF_TILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < IF_TILE + 2; q += IF_TS) {
      const bool ok = t0 + q < s1;
      IStation z = {0.f, 0.f, 0.f, 0.f};
      const IStation f = ok ? sf[t0 + q] : z;
      const int2 h = ok ? si[t0 + q] : make_int2(0, 0);
      s_ex[q] = f.ex;
      s_ey[q] = f.ey;
      s_zs[q] = f.zs;
      s_r[q] = f.r;
      s_hx[q] = (float)h.x;
      s_hy[q] = (float)h.y;
      s_i[q] = h;
      s_nf[q] = ok ? anynear[t0 + q] : 0;
    }
    __syncthreads();
    if (!active) continue;
    const int cnt = min(IF_TILE, s1 - t0);
    float2 gr = make_float2(0.f, 0.f), gd = make_float2(0.f, 0.f);  // 32 stations, Kahan across
#pragma unroll 4
    for (int q = 0; q < cnt; q += 2) {
      // stations q and q+1 (the second is dropped past the end of the tile)
      const float2 hx = *reinterpret_cast<const float2*>(s_hx + q);
      const float2 hy = *reinterpret_cast<const float2*>(s_hy + q);
      const float2 X = __ffma2_rn(__fadd2_rn(hx, nix2), dxn2,
                                  *reinterpret_cast<const float2*>(s_ex + q));
      const float2 Y = __ffma2_rn(__fadd2_rn(hy, niy2), dyn2,
                                  *reinterpret_cast<const float2*>(s_ey + q));
      const float2 X2 = __fmul2_rn(X, X), Y2 = __fmul2_rn(Y, Y), rh = __fadd2_rn(X2, Y2);
      const float2 ut = __fadd2_rn(*reinterpret_cast<const float2*>(s_zs + q), cy2);
      const float2 rt2 = __ffma2_rn(ut, ut, rh);
      float2 itop, u, f;
      // second order when every lane's pairs are far enough (warp-uniform)
      if (__all_sync(__activemask(), fminf(rt2.x, rt2.y) >= k.rt2_t2)) {
        u = col_unit2<true>(X2, Y2, rh, ut, rt2, cz2, k, &itop);
        f = face_unit_far2<true>(X2, Y2, ut, itop, k.face);
      } else {
        u = col_unit2<false>(X2, Y2, rh, ut, rt2, cz2, k, &itop);
        f = face_unit_far2<false>(X2, Y2, ut, itop, k.face);
      }
      const float2 r = *reinterpret_cast<const float2*>(s_r + q);
      float2 vr = __fmul2_rn(r, u), vd = __fmul2_rn(r, f);
      // near pairs go through the double path: select, which also drops a
      // NaN.  Every lane has the same stations, so the test is uniform.
      if (s_nf[q] | s_nf[q + 1]) {
        const int2 ha = s_i[q], hb = s_i[q + 1];
        if (is_near(mask, t0 + q, ha.x, ha.y, ix, iy, k)) vr.x = vd.x = 0.f;
        if (q + 1 < cnt && is_near(mask, t0 + q + 1, hb.x, hb.y, ix, iy, k)) vr.y = vd.y = 0.f;
      }
      if (q + 1 >= cnt) vr.y = vd.y = 0.f;  // the padding station
      gr = __fadd2_rn(gr, vr);
      gd = __fadd2_rn(gd, vd);
      if ((q & 30) == 30) {
        ar.add(gr.x + gr.y);
        ad.add(gd.x + gd.y);
        gr = gd = make_float2(0.f, 0.f);
      }
    }
    ar.add(gr.x + gr.y);
    ad.add(gd.x + gd.y);
  }
  if (!active) return;
  const size_t o = (size_t)blockIdx.y * k.ncols + c;
  p_rho[o] = ar.value();
  p_dep[o] = (double)col.x * ad.value();
}

// g_rho[c] = sc_rho * sum_chunks p_rho,  g_dep[c] = -sc_dep * sum_chunks p_dep
// (fixed order: bitwise reproducible for a launch shape)
__global__ void iface_far_adj_finalize(long long nc, int nchunks, const double* __restrict__ p_rho,
                                       const double* __restrict__ p_dep, double sc_rho,
                                       double sc_dep, double* __restrict__ g_rho,
                                       double* __restrict__ g_dep) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double r = 0.0, d = 0.0;
  for (int q = 0; q < nchunks; q++) {
    r += p_rho[(size_t)q * nc + c];
    d += p_dep[(size_t)q * nc + c];
  }
  if (g_rho) g_rho[c] = sc_rho * r;
  if (g_dep) g_dep[c] = -sc_dep * d;
}

// ---- adjoint, near window in double (warp per station, atomics) ------------
__global__ void iface_near_adj(IConst k, IMeshDesc m, int ns, const double* __restrict__ sxyz,
                               const int2* __restrict__ si, const double* __restrict__ depth,
                               const double* __restrict__ rho, const double* __restrict__ res,
                               const uint32_t* __restrict__ mask, double G5,
                               double* __restrict__ g_rho, double* __restrict__ g_dep) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * IF_NEAR_WPB + warp;
  if (s >= ns) return;
  const double r = res[s];
  if (r == 0.0) return;
  const int2 h = si[s];
  const int cx = clampi(h.x, 0, k.nx - 1), cy = clampi(h.y, 0, k.ny - 1);
  const int x0 = max(0, cx - k.w), x1 = min(k.nx - 1, cx + k.w);
  const int y0 = max(0, cy - k.w), y1 = min(k.ny - 1, cy + k.w);
  const int wx = x1 - x0 + 1, n = wx * (y1 - y0 + 1);
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  for (int q = lane; q < n; q += 32) {
    if (!((mask[(size_t)s * k.words + (q >> 5)] >> (q & 31)) & 1u)) continue;
    const int ix = x0 + q % wx, iy = y0 + q / wx;
    const long long c = ix + (long long)m.nx * iy;
    const double xa = (m.x0 + ix * m.dx) - xs, xb = (m.x0 + (ix + 1) * m.dx) - xs;
    const double ya = (m.y0 + iy * m.dy) - ys, yb = (m.y0 + (iy + 1) * m.dy) - ys;
    const double ztop = -depth[c];
    if (g_rho) {
      double u = ztm_prism_unit<double>(xa, xb, ya, yb, m.zb - zs, ztop - zs);
      atomicAdd(&g_rho[c], G5 * r * u);
    }
    if (g_dep) {
      double f = ztm_face_unit(xa, xb, ya, yb, zs - ztop);
      atomicAdd(&g_dep[c], -G5 * rho[c] * r * f);
    }
  }
}

// ---- adjoint, plain double (thread per column, station chunks) --------------
__global__ void __launch_bounds__(IF_TS)
    iface_f64_adj(IMeshDesc m, int ns, const double* __restrict__ sxyz,
                  const double* __restrict__ depth, const double* __restrict__ res, int chunk_len,
                  double* __restrict__ pr, double* __restrict__ pd) {
  const long long nc = (long long)m.nx * m.ny;
  const long long c = blockIdx.x * (long long)IF_TS + threadIdx.x;
  if (c >= nc) return;
  const int ix = (int)(c % m.nx), iy = (int)(c / m.nx);
  const double ztop = -depth[c];
  const int s0 = blockIdx.y * chunk_len, s1 = min(ns, s0 + chunk_len);
  double ar = 0.0, ad = 0.0;
  for (int s = s0; s < s1; s++) {
    const double r = res[s];
    if (r == 0.0) continue;
    const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
    const double xa = (m.x0 + ix * m.dx) - xs, xb = (m.x0 + (ix + 1) * m.dx) - xs;
    const double ya = (m.y0 + iy * m.dy) - ys, yb = (m.y0 + (iy + 1) * m.dy) - ys;
    if (pr) ar += r * ztm_prism_unit<double>(xa, xb, ya, yb, m.zb - zs, ztop - zs);
    if (pd) ad += r * ztm_face_unit(xa, xb, ya, yb, zs - ztop);
  }
  if (pr) pr[(size_t)blockIdx.y * nc + c] = ar;
  if (pd) pd[(size_t)blockIdx.y * nc + c] = ad;
}

__global__ void iface_f64_adj_finalize(long long nc, int nchunks, const double* __restrict__ pr,
                                       const double* __restrict__ pd,
                                       const double* __restrict__ rho, double G5,
                                       double* __restrict__ g_rho, double* __restrict__ g_dep) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nchunks; k++) {
    if (pr) a += pr[(size_t)k * nc + c];
    if (pd) b += pd[(size_t)k * nc + c];
  }
  if (g_rho) g_rho[c] = G5 * a;
  if (g_dep) g_dep[c] = -G5 * rho[c] * b;
}

// residual and misfit: r = gz - data, misfit = 0.5 * sum r^2 (one block,
// fixed reduction order).
__global__ void residual_kernel(int ns, const double* __restrict__ gz,
                                const double* __restrict__ data, double* __restrict__ r,
                                double* __restrict__ misfit) {
  __shared__ double red[1024];
  double a = 0.0;
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    double v = gz[s] - data[s];
    r[s] = v;
    a += v * v;
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *misfit = 0.5 * red[0];
}

int chunks_for(long long units, int tiles, int num_sms, int minlen, int* len, int per_sm = 8) {
  long long want = std::max(1LL, ((long long)per_sm * std::max(num_sms, 1)) / std::max(tiles, 1));
  long long ch = std::min<long long>(want, std::max(1LL, units / minlen));
  ch = std::max(1LL, std::min(ch, 65535LL));
  *len = (int)((units + ch - 1) / ch);
  if (*len < 1) *len = 1;
  return (int)((units + *len - 1) / *len);
}

// Station slices of the mixed adjoint: about twelve waves of blocks of
// column tiles x slices (blocks finish unevenly; three waves left the end of
// the launch half idle), slices of at least one shared-memory tile.
int iface_adj_chunks(int ns, long long nc, int num_sms, int* len) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, iface_far_adj, IF_TS, 0) != cudaSuccess ||
      occ < 1) {
    cudaGetLastError();
    occ = 1;
  }
  const long long tiles = std::max(1LL, (nc + IF_TS - 1) / IF_TS);
  long long ch = std::max(1LL, 12LL * occ * std::max(num_sms, 1) / tiles);
  ch = std::min(ch, std::max(1LL, (long long)(ns + IF_TILE - 1) / IF_TILE));
  ch = std::min(ch, 65535LL);
  *len = (int)((std::max(ns, 1) + ch - 1) / ch);
  return (int)((std::max(ns, 1) + *len - 1) / *len);
}

}  // namespace

size_t ztm_iface_ws(const IMeshDesc& m, int ns, int precision, int num_sms) {
  long long nc = (long long)m.nx * m.ny;
  int len;
  int tiles = std::max(1, (ns + 63) / 64);
  int ch = chunks_for(nc, tiles, num_sms, 64, &len);
  ch = std::max(ch, chunks_for(nc, std::max(1, (ns + IF_TS - 1) / IF_TS), num_sms, IF_TILE, &len,
                               IF_FWD_PER_SM));
  int cha = chunks_for(std::max(ns, 1), (int)((nc + IF_TS - 1) / IF_TS), num_sms, 32, &len);
  size_t w = WsCarver::need((size_t)ch * std::max(ns, 1) * 8) * 2;  // forward partials (x2 slack)
  w += WsCarver::need((size_t)cha * nc * 8) * 2;                    // double adjoint partials
  const int chm = iface_adj_chunks(ns, nc, num_sms, &len);
  w += WsCarver::need((size_t)chm * nc * 8) * 2;                    // mixed adjoint partials
  // a second set of station and column arrays (forward + adjoint in one call)
  w += WsCarver::need((size_t)nc * 16) + WsCarver::need((size_t)std::max(ns, 1) * 24);
  w += WsCarver::need((size_t)nc * 16) + WsCarver::need((size_t)std::max(ns, 1) * 16) +
       WsCarver::need((size_t)std::max(ns, 1) * 8) * 4;
  // near masks (forward and adjoint), up to near_q = 16
  w += 2 * WsCarver::need((size_t)std::max(ns, 1) * 4 * 64);
  // per-station "has a near column" flags (forward and adjoint)
  w += 2 * WsCarver::need((size_t)std::max(ns, 1) * 4);
  // the forward's station order (and the sort's scratch), twice for slack
  w += 2 * (WsCarver::need((size_t)std::max(ns, 1) * 4) + ztm_station_order_ws(ns, m.nx, m.ny));
  (void)precision;
  return w;
}

// The forward (vdep == nullptr) or the depth directional derivative
// dgz[s] = sum_c dgz[s]/ddepth[c] vdep[c] = -G5 rho_c * (top-face integral):
// the same kernels with the face integral in place of the column integral
// and the columns weighted by rho * vdep.
template <bool FACE>
static int iface_forward_impl(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                              const double* d_rho, const double* d_vdep, int ns,
                              const double* d_sxyz, double* d_gz, double G, int precision,
                              const ztm_opts* o, WsCarver& wc) {
  const double G5 = G * 1.0e5;
  const double sign = FACE ? -1.0 : 1.0;
  const long long nc = (long long)m.nx * m.ny;
  if (precision == ZTM_PREC_FP64) {
    int tiles = std::max(1, (ns + 63) / 64), len;
    int ch = chunks_for(nc, tiles, c->num_sms, 64, &len);
    double* partial = wc.take<double>((size_t)ch * ns);
    {
      ZtmProf prof_(c, "iface_f64");
      iface_f64_fwd<FACE><<<dim3(tiles, ch), 64, 0, c->stream>>>(m, ns, d_sxyz, d_depth, d_rho,
                                                                 d_vdep, len, partial);
    }
    iface_finalize<<<(ns + 255) / 256, 256, 0, c->stream>>>(ns, ch, partial, 1.0, nullptr,
                                                            sign * G5, d_gz);
    c->launches += 2;
    return ztm_after_launch(c, "interface FP64 kernels");
  }
  const double nq = (o && o->near_q > 0) ? o->near_q : 6.0;
  IConst k = make_iconst(m, nq);
  if (k.words > 64) return ztm_fail(c, ZTM_ERR_RANGE, "near_q too large for the interface window");
  IStation* sf = wc.take<IStation>(ns);
  int2* si = wc.take<int2>(ns);
  float4* cf = wc.take<float4>(nc);
  double* near = wc.take<double>(ns);
  iface_station_prep<<<(ns + 127) / 128, 128, 0, c->stream>>>(m, k.L0, ns, d_sxyz, nullptr, sf,
                                                              si);
  int* perm = wc.take<int>(ns);
  if (int rc = ztm_station_order(c, c->stream, ns, reinterpret_cast<const int*>(si), 2, m.nx, m.ny,
                                 perm, wc))
    return rc;
  iface_col_prep<<<(unsigned)((nc + 255) / 256), 256, 0, c->stream>>>(m, k.L0, d_depth, d_rho,
                                                                   FACE ? d_vdep : nullptr, cf);
  uint32_t* mask = wc.take<uint32_t>((size_t)ns * k.words);
  int* anynear = wc.take<int>((size_t)ns);
  iface_near_mask<<<(ns + 3) / 4, 128, 0, c->stream>>>(k, ns, d_sxyz, si, d_depth, mask, anynear);
  // double near columns on the side stream, concurrently with the float far field
  ztm_fork(c);
  {
    ZtmProf prof_(c, "iface_near", c->aux);
    iface_near_fwd<FACE><<<(ns + IF_NEAR_WPB - 1) / IF_NEAR_WPB, IF_NEAR_WPB * 32, 0, c->aux>>>(
        k, m, ns, d_sxyz, si, d_depth, d_rho, d_vdep, mask, near);
  }
  int tiles = std::max(1, (ns + IF_TS - 1) / IF_TS), len;
  int ch = chunks_for(nc, tiles, c->num_sms, IF_TILE, &len, IF_FWD_PER_SM);
  double* partial = wc.take<double>((size_t)ch * ns);
  {
    ZtmProf prof_(c, "iface_far");
    iface_far_fwd<FACE><<<dim3(tiles, ch), IF_TS, 0, c->stream>>>(k, ns, sf, si, cf, mask,
                                                                  anynear, perm, len, partial);
  }
  ztm_join(c);
  // the column integral is in units of L0 (x dx dy / L0^2), the face
  // integral is dimensionless (x dx dy / L0^2)
  const double far_scale = (FACE ? 1.0 : k.L0) * (double)k.dxn * k.dyn;
  iface_finalize<<<(ns + 255) / 256, 256, 0, c->stream>>>(ns, ch, partial, far_scale, near,
                                                          sign * G5, d_gz);
  c->launches += 6;
  return ztm_after_launch(c, "interface mixed kernels");
}

int ztm_launch_iface_fwd(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, int ns, const double* d_sxyz, double* d_gz,
                         double G, int precision, const ztm_opts* o, WsCarver& wc) {
  return iface_forward_impl<false>(c, m, d_depth, d_rho, nullptr, ns, d_sxyz, d_gz, G, precision,
                                   o, wc);
}

int ztm_launch_iface_jvp(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, const double* d_vdep, int ns, const double* d_sxyz,
                         double* d_dgz, double G, int precision, const ztm_opts* o,
                         WsCarver& wc) {
  return iface_forward_impl<true>(c, m, d_depth, d_rho, d_vdep, ns, d_sxyz, d_dgz, G, precision,
                                  o, wc);
}

int ztm_launch_iface_adj(ztm_ctx* c, const IMeshDesc& m, const double* d_depth,
                         const double* d_rho, int ns, const double* d_sxyz, const double* d_res,
                         double* d_grho, double* d_gdep, double G, int precision,
                         const ztm_opts* o, WsCarver& wc) {
  const double G5 = G * 1.0e5;
  const long long nc = (long long)m.nx * m.ny;
  if (ns == 0) {
    if (d_grho) cudaMemsetAsync(d_grho, 0, nc * 8, c->stream);
    if (d_gdep) cudaMemsetAsync(d_gdep, 0, nc * 8, c->stream);
    return ztm_after_launch(c, "interface adjoint (no stations)");
  }
  if (precision == ZTM_PREC_FP64) {
    int len;
    int ch = chunks_for(ns, (int)((nc + IF_TS - 1) / IF_TS), c->num_sms, 32, &len);
    double* pr = d_grho ? wc.take<double>((size_t)ch * nc) : nullptr;
    double* pd = d_gdep ? wc.take<double>((size_t)ch * nc) : nullptr;
    {
      ZtmProf prof_(c, "iface_f64");
      iface_f64_adj<<<dim3((unsigned)((nc + IF_TS - 1) / IF_TS), ch), IF_TS, 0, c->stream>>>(
          m, ns, d_sxyz, d_depth, d_res, len, pr, pd);
    }
    iface_f64_adj_finalize<<<(unsigned)((nc + 255) / 256), 256, 0, c->stream>>>(
        nc, ch, pr, pd, d_rho, G5, d_grho, d_gdep);
    c->launches += 2;
    return ztm_after_launch(c, "interface FP64 adjoint");
  }
  const double nq = (o && o->near_q > 0) ? o->near_q : 6.0;
  IConst k = make_iconst(m, nq);
  if (k.words > 64) return ztm_fail(c, ZTM_ERR_RANGE, "near_q too large for the interface window");
  IStation* sf = wc.take<IStation>(ns);
  int2* si = wc.take<int2>(ns);
  float4* cf = wc.take<float4>(nc);
  iface_station_prep<<<(ns + 127) / 128, 128, 0, c->stream>>>(m, k.L0, ns, d_sxyz, d_res, sf, si);
  iface_col_prep<<<(unsigned)((nc + 255) / 256), 256, 0, c->stream>>>(m, k.L0, d_depth, d_rho,
                                                                   nullptr, cf);
  // face integral is dimensionless: dx dy / L0^2 * (u / r^3 in 1/L0^2 units)
  const double sc_rho = G5 * k.L0 * (double)k.dxn * k.dyn;
  const double sc_dep = G5 * (double)k.dxn * k.dyn;
  uint32_t* mask = wc.take<uint32_t>((size_t)ns * k.words);
  int* anynear = wc.take<int>((size_t)ns);
  iface_near_mask<<<(ns + 3) / 4, 128, 0, c->stream>>>(k, ns, d_sxyz, si, d_depth, mask, anynear);
  int alen;
  const int ach = iface_adj_chunks(ns, nc, c->num_sms, &alen);
  double* p_rho = wc.take<double>((size_t)ach * nc);
  double* p_dep = wc.take<double>((size_t)ach * nc);
  {
    ZtmProf prof_(c, "iface_far");
    iface_far_adj<<<dim3((unsigned)((nc + IF_TS - 1) / IF_TS), ach), IF_TS, 0, c->stream>>>(
        k, ns, sf, si, cf, mask, anynear, alen, p_rho, p_dep);
  }
  iface_far_adj_finalize<<<(unsigned)((nc + 255) / 256), 256, 0, c->stream>>>(
      nc, ach, p_rho, p_dep, sc_rho, sc_dep, d_grho, d_gdep);
  {  // after the far kernel has written every entry: double atomics add the near pairs
    ZtmProf prof_(c, "iface_near");
    iface_near_adj<<<(ns + IF_NEAR_WPB - 1) / IF_NEAR_WPB, IF_NEAR_WPB * 32, 0, c->stream>>>(
        k, m, ns, d_sxyz, si, d_depth, d_rho, d_res, mask, G5, d_grho, d_gdep);
  }
  c->launches += 6;
  return ztm_after_launch(c, "interface mixed adjoint");
}

// ---------------------------------------------------------------------------
// forward + misfit + adjoint (C ABI)
extern "C" int ztm_gfm_interface_misfit(ztm_ctx* c, const ztm_imesh* mesh, const double* depth,
                                        const double* rho_col, int ns, const double* sxyz,
                                        const double* data, double* misfit, double* gz,
                                        double* g_rho, double* g_depth, const ztm_opts* o) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!mesh || !depth || !rho_col || !sxyz || !data || !misfit)
    return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (mesh->nx < 1 || mesh->ny < 1 || !(mesh->dx > 0) || !(mesh->dy > 0))
    return ztm_fail(c, ZTM_ERR_ARG, "bad interface mesh");
  if (ns < 1) return ztm_fail(c, ZTM_ERR_ARG, "ns must be >= 1");
  if (o && (o->precision < 0 || o->precision > 2 || (o->flags & ~ZTM_FLAG_DEVICE_PTRS)))
    return ztm_fail(c, ZTM_ERR_ARG, "bad options");
  const int prec = o ? o->precision : ZTM_PREC_FP64;
  const bool dev = o && (o->flags & ZTM_FLAG_DEVICE_PTRS);
  const double G = (o && o->G > 0) ? o->G : 6.67e-11;
  IMeshDesc m;
  m.nx = mesh->nx; m.ny = mesh->ny; m.x0 = mesh->x0; m.y0 = mesh->y0;
  m.dx = mesh->dx; m.dy = mesh->dy; m.zb = mesh->z_base;
  const long long nc = (long long)m.nx * m.ny;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device) cudaSetDevice(c->device);
  struct Restore {
    int p, d;
    ~Restore() {
      if (p >= 0 && p != d) cudaSetDevice(p);
    }
  } restore{prev, c->device};
  size_t need = 2 * WsCarver::need(nc * 8) + WsCarver::need((size_t)ns * 24) +
                4 * WsCarver::need((size_t)ns * 8) + 2 * WsCarver::need(nc * 8) + 256 +
                ztm_iface_ws(m, ns, prec, c->num_sms) + 4096;
  int rc = ztm_ws_reserve(c, need);
  if (rc) return rc;
  WsCarver wc(c->ws);
  double* s_dep = wc.take<double>(nc);
  double* s_rho = wc.take<double>(nc);
  double* s_xyz = wc.take<double>((size_t)ns * 3);
  double* s_dat = wc.take<double>(ns);
  double* s_gz = wc.take<double>(ns);
  double* s_r = wc.take<double>(ns);
  double* s_mis = wc.take<double>(1);
  double* s_gr = wc.take<double>(nc);
  double* s_gd = wc.take<double>(nc);
  const void *pd, *pr, *px, *pdat;
  if ((rc = ztm_stage_in(c, depth, nc * 8, dev, s_dep, &pd))) return rc;
  if ((rc = ztm_stage_in(c, rho_col, nc * 8, dev, s_rho, &pr))) return rc;
  if ((rc = ztm_stage_in(c, sxyz, (size_t)ns * 24, dev, s_xyz, &px))) return rc;
  if ((rc = ztm_stage_in(c, data, (size_t)ns * 8, dev, s_dat, &pdat))) return rc;
  double* ogz = (dev && gz) ? gz : s_gz;
  rc = iface_forward_impl<false>(c, m, (const double*)pd, (const double*)pr, nullptr, ns,
                                 (const double*)px, ogz,
                          G, prec, o, wc);
  if (rc) return rc;
  double* omis = dev ? misfit : s_mis;
  residual_kernel<<<1, 1024, 0, c->stream>>>(ns, ogz, (const double*)pdat, s_r, omis);
  c->launches++;
  double* ogr = g_rho ? (dev ? g_rho : s_gr) : nullptr;
  double* ogd = g_depth ? (dev ? g_depth : s_gd) : nullptr;
  if (ogr || ogd) {
    rc = ztm_launch_iface_adj(c, m, (const double*)pd, (const double*)pr, ns, (const double*)px,
                              s_r, ogr, ogd, G, prec, o, wc);
    if (rc) return rc;
  }
  if ((rc = ztm_cuda_check(c, cudaGetLastError(), "interface misfit kernels"))) return rc;
  if (dev) return ZTM_OK;
  cudaMemcpyAsync(misfit, s_mis, 8, cudaMemcpyDeviceToHost, c->stream);
  if (gz) cudaMemcpyAsync(gz, s_gz, (size_t)ns * 8, cudaMemcpyDeviceToHost, c->stream);
  if (g_rho) cudaMemcpyAsync(g_rho, s_gr, nc * 8, cudaMemcpyDeviceToHost, c->stream);
  if (g_depth) cudaMemcpyAsync(g_depth, s_gd, nc * 8, cudaMemcpyDeviceToHost, c->stream);
  if ((rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "interface misfit"))) return rc;
  return ztm_check_device_error(c);
}
