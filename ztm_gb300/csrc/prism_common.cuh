// prism_common.cuh - geometry preparation and the far-field expansion shared
// by the forward, adjoint and batched prism kernels.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "ztm_internal.cuh"

// Far-field expansion of one prism's attraction, relative to the point-mass
// term.  With (X, Y, Z) = station minus prism centre and r = |(X,Y,Z)|:
//   gz = G rho V Z/r^3 * [1 + t2 + t4 + t6],
//   t2 = (cA X^2 + cB Y^2 + a1 Z^2) / r^4,
//   t4 = (h0 + h1 Z^2 + h2 Z^4) / r^8,
//   h1 = cX1 X^2 + cY1 Y^2,  h0 = cXX X^4 + cXY X^2 Y^2 + cYY Y^4,
//   t6 = (k0 + k1 Z^2 + k2 Z^4 + k3 Z^6) / r^12,
//   k2 = kX2 X^2 + kY2 Y^2,  k1 = kXX X^4 + kXY X^2 Y^2 + kYY Y^4,
//   k0 = kX3 X^6 + kX2Y X^4 Y^2 + kXY2 X^2 Y^4 + kY3 Y^6.
// This is the Taylor expansion of Z/r^3 over the prism volume to sixth
// order: the average over the box of the derivatives times the moments
// (a^2n/(2n+1) for a half edge a, products for mixed terms; odd moments
// vanish by symmetry), each order gathered over r^(2p).  The coefficients
// were derived symbolically; the second and fourth orders are those of the
// classic moment expansion (second moments dx^2/12, fourth dx^4/80, mixed
// dx^2 dy^2/144).  Beyond 4 half-diagonals the sixth-order form is within
// about 4e-7 of the closed form (relative to V/r^2; the fourth-order form
// reaches that only beyond 6).  Lengths are in the normalised unit L0 (the
// largest cell edge) so that float cannot overflow.
struct FarCoef {
  float cA, cB, a1;
  float cX1, cY1, cXX, cXY, cYY, h2;
  float k3, kX2, kY2, kXX, kXY, kYY, kX3, kX2Y, kXY2, kY3;
};

__host__ __device__ inline FarCoef far_coef(double dx, double dy, double dz) {
  double x2 = dx * dx, y2 = dy * dy, z2 = dz * dz;
  double x4 = x2 * x2, y4 = y2 * y2, z4 = z2 * z2;
  FarCoef f;
  f.cA = (float)((4 * x2 - y2 - 3 * z2) / 8);
  f.cB = (float)((4 * y2 - x2 - 3 * z2) / 8);
  f.a1 = (float)((2 * z2 - x2 - y2) / 8);
  f.h2 = (float)((9 * x4 + 10 * x2 * y2 - 40 * x2 * z2 + 9 * y4 - 40 * y2 * z2 + 24 * z4) / 384);
  f.cX1 = (float)(-(54 * x4 + 25 * x2 * y2 - 205 * x2 * z2 - 9 * y4 + 5 * y2 * z2 + 60 * z4) / 192);
  f.cY1 = (float)(-(-9 * x4 + 25 * x2 * y2 + 5 * x2 * z2 + 54 * y4 - 205 * y2 * z2 + 60 * z4) / 192);
  f.cXX = (float)((24 * x4 - 20 * x2 * y2 - 60 * x2 * z2 + 3 * y4 + 10 * y2 * z2 + 15 * z4) / 128);
  f.cXY = (float)((-36 * x4 + 170 * x2 * y2 - 50 * x2 * z2 - 36 * y4 - 50 * y2 * z2 + 30 * z4) / 128);
  f.cYY = (float)((3 * x4 - 20 * x2 * y2 + 10 * x2 * z2 + 24 * y4 - 60 * y2 * z2 + 15 * z4) / 128);
  double x6 = x4 * x2, y6 = y4 * y2, z6 = z4 * z2;
  f.k3 = (float)((-15 * x6 - 21 * x4 * y2 + 126 * x4 * z2 - 21 * x2 * y4 + 140 * x2 * y2 * z2 -
                  168 * x2 * z4 - 15 * y6 + 126 * y4 * z2 - 168 * y2 * z4 + 48 * z6) / 3072);
  f.kX2 = (float)((120 * x6 + 105 * x4 * y2 - 945 * x4 * z2 + 42 * x2 * y4 - 490 * x2 * y2 * z2 +
                   1092 * x2 * z4 - 15 * y6 + 63 * y4 * z2 + 84 * y2 * z4 - 168 * z6) / 1024);
  f.kY2 = (float)((-15 * x6 + 42 * x4 * y2 + 63 * x4 * z2 + 105 * x2 * y4 - 490 * x2 * y2 * z2 +
                   84 * x2 * z4 + 120 * y6 - 945 * y4 * z2 + 1092 * y2 * z4 - 168 * z6) / 1024);
  f.kXX = (float)((-240 * x6 + 1680 * x4 * z2 + 105 * x2 * y4 - 350 * x2 * y2 * z2 -
                   1575 * x2 * z4 - 15 * y6 + 105 * y2 * z4 + 210 * z6) / 1024);
  f.kXY = (float)((120 * x6 - 525 * x4 * y2 - 315 * x4 * z2 - 525 * x2 * y4 + 3500 * x2 * y2 * z2 -
                   735 * x2 * z4 + 120 * y6 - 315 * y4 * z2 - 735 * y2 * z4 + 210 * z6) / 512);
  f.kYY = (float)((-15 * x6 + 105 * x4 * y2 - 350 * x2 * y2 * z2 + 105 * x2 * z4 - 240 * y6 +
                   1680 * y4 * z2 - 1575 * y2 * z4 + 210 * z6) / 1024);
  f.kX3 = (float)((192 * x6 - 336 * x4 * y2 - 1008 * x4 * z2 + 168 * x2 * y4 + 560 * x2 * y2 * z2 +
                   840 * x2 * z4 - 15 * y6 - 63 * y4 * z2 - 105 * y2 * z4 - 105 * z6) / 3072);
  f.kX2Y = (float)((-240 * x6 + 1680 * x4 * y2 - 1155 * x2 * y4 - 1750 * x2 * y2 * z2 +
                    525 * x2 * z4 + 120 * y6 + 315 * y4 * z2 + 210 * y2 * z4 - 105 * z6) / 1024);
  f.kXY2 = (float)((120 * x6 - 1155 * x4 * y2 + 315 * x4 * z2 + 1680 * x2 * y4 - 1750 * x2 * y2 * z2 +
                    210 * x2 * z4 - 240 * y6 + 525 * y2 * z4 - 105 * z6) / 1024);
  f.kY3 = (float)((-15 * x6 + 168 * x4 * y2 - 63 * x4 * z2 - 336 * x2 * y4 + 560 * x2 * y2 * z2 -
                   105 * x2 * z4 + 192 * y6 - 1008 * y4 * z2 + 840 * y2 * z4 - 105 * z6) / 3072);
  return f;
}

// Per-(station, column) coefficients of the far-field correction written
// as a polynomial in u = 1/r^2: substituting Z^2 = r^2 - rh (rh = X^2+Y^2)
// into t2 + t4 + t6 gives
//   1 + t2 + t4 + t6 = 1 + u (a1 + u (C2 + u (C3 + u (C4 + u (C5 + u C6))))),
//   C2 = a0 - a1 rh + h2,  C3 = h1 - 2 h2 rh + k3,
//   C4 = h0 - h1 rh + h2 rh^2 + k2 - 3 k3 rh,
//   C5 = k1 - 2 k2 rh + 3 k3 rh^2,  C6 = k0 - k1 rh + k2 rh^2 - k3 rh^3,
// so a pair costs one rsqrt and a 6-term Horner chain, with no Z^2 terms.
struct ColPoly {
  float rh, C2, C3, C4, C5, C6;
};

__device__ __forceinline__ ColPoly col_poly(float X, float Y, const FarCoef& f) {
  const float X2 = X * X, Y2 = Y * Y, rh = X2 + Y2;
  const float a0 = fmaf(X2, f.cA, Y2 * f.cB);
  const float h1 = fmaf(X2, f.cX1, Y2 * f.cY1);
  const float h0 = fmaf(X2, fmaf(X2, f.cXX, Y2 * f.cXY), Y2 * Y2 * f.cYY);
  const float k2 = fmaf(X2, f.kX2, Y2 * f.kY2);
  const float k1 = fmaf(X2, fmaf(X2, f.kXX, Y2 * f.kXY), Y2 * Y2 * f.kYY);
  const float k0 = fmaf(X2, fmaf(X2, fmaf(X2, f.kX3, Y2 * f.kX2Y), Y2 * Y2 * f.kXY2),
                        Y2 * Y2 * Y2 * f.kY3);
  ColPoly c;
  c.rh = rh;
  c.C2 = fmaf(-f.a1, rh, a0) + f.h2;
  c.C3 = fmaf(-2.f * f.h2, rh, h1) + f.k3;
  c.C4 = fmaf(fmaf(f.h2, rh, -h1), rh, h0) + fmaf(-3.f * f.k3, rh, k2);
  c.C5 = fmaf(fmaf(3.f * f.k3, rh, -2.f * k2), rh, k1);
  c.C6 = fmaf(fmaf(fmaf(-f.k3, rh, k2), rh, -k1), rh, k0);
  return c;
}

// Reciprocal square root on the special-function unit, subnormals flushed
// (PTX rsqrt.approx.ftz.f32): far-field distances are never subnormal, and
// the flush spares the scaling steps an IEEE-subnormal-safe rsqrtf needs.
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Two layers at once on the packed FP32 path (Blackwell FFMA2/FMUL2: one
// issue slot for two float FMAs with the same rounding as two FFMAs); the
// two rsqrts stay scalar on the special-function unit.  Returns
// (Z/r^3 (1+t2+t4)) for Z = Zv.x and Zv.y.
struct ColPoly2 {
  float2 rh, C2, C3, C4, C5, C6, a1;
};

__device__ __forceinline__ ColPoly2 col_poly2(const ColPoly& c, float a1) {
  ColPoly2 d;
  d.rh = make_float2(c.rh, c.rh);
  d.C2 = make_float2(c.C2, c.C2);
  d.C3 = make_float2(c.C3, c.C3);
  d.C4 = make_float2(c.C4, c.C4);
  d.C5 = make_float2(c.C5, c.C5);
  d.C6 = make_float2(c.C6, c.C6);
  d.a1 = make_float2(a1, a1);
  return d;
}

__device__ __forceinline__ float2 far_unit2(float2 Z, const ColPoly2& c) {
  const float2 r2 = __ffma2_rn(Z, Z, c.rh);
  const float2 rinv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
  const float2 u = __fmul2_rn(rinv, rinv);
  float2 p = __ffma2_rn(c.C6, u, c.C5);
  p = __ffma2_rn(p, u, c.C4);
  p = __ffma2_rn(p, u, c.C3);
  p = __ffma2_rn(p, u, c.C2);
  p = __ffma2_rn(p, u, c.a1);
  const float2 s = __ffma2_rn(p, u, make_float2(1.f, 1.f));
  return __fmul2_rn(__fmul2_rn(Z, s), __fmul2_rn(rinv, u));
}

// Second-order form for pairs at least 48 half-diagonals away (horizontal
// distance alone): 1 + t2 = 1 + u (a1 + u C2t), C2t = a0 - a1 rh.  The
// dropped fourth-order term is below 2e-8 of the pair's monopole there.
__device__ __forceinline__ float2 far_unit2_t2(float2 Z, const ColPoly2& c, float2 C2t) {
  const float2 r2 = __ffma2_rn(Z, Z, c.rh);
  const float2 rinv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
  const float2 u = __fmul2_rn(rinv, rinv);
  const float2 p = __ffma2_rn(C2t, u, c.a1);
  const float2 s = __ffma2_rn(p, u, make_float2(1.f, 1.f));
  return __fmul2_rn(__fmul2_rn(Z, s), __fmul2_rn(rinv, u));
}

// Default near radius of the 3-D mesh's mixed kernels, in prism
// half-diagonals: beyond it the sixth-order far field is within about 4e-7
// of the closed form (relative to V/r^2), as the fourth-order form was only
// beyond 6.
constexpr double ZTM_MESH_NEAR_Q = 4.0;

// Regular-mesh constants for the mixed kernels.
struct MeshConst {
  int nx, ny, nz, nzp;  // nzp: layers padded to a multiple of 8
  int ncols;
  int wx, wy, wl;       // near-box half widths (columns, columns, layers)
  float dxn, dyn, dzn;  // cell edges / L0
  float rh_t2;          // horizontal distance^2 (units of L0) beyond which
                        // the second-order form is exact enough
  double L0;
  double dxm, dym, dzm;  // cell edges (m)
  double R2;             // (near_q * half diagonal)^2 (m^2)
  int nslots;            // (2wx+1)(2wy+1): columns of a near box
  FarCoef fc;
};

// Half widths of the near box: every prism outside it has its centre at
// least near_q * (half diagonal) from the station.  A prism whose index
// differs from the station's home index by k >= w+1 along an axis is at
// least (w + 1/2) cells away along that axis.
inline void near_widths(double dx, double dy, double dz, double near_q, int* wx, int* wy,
                        int* wl) {
  double ell = 0.5 * sqrt(dx * dx + dy * dy + dz * dz);
  double R = near_q * ell;
  *wx = (int)ceil(R / dx - 0.5);
  *wy = (int)ceil(R / dy - 0.5);
  *wl = (int)ceil(R / dz - 0.5);
  if (*wx < 0) *wx = 0;
  if (*wy < 0) *wy = 0;
  if (*wl < 0) *wl = 0;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

// Near box of a station (inclusive bounds), clamped to the mesh.
struct NearBox {
  int x0, x1, y0, y1, l0, l1;
};
__device__ __forceinline__ NearBox near_box(int4 si, const MeshConst& k) {
  NearBox b;
  int cx = clampi(si.x, 0, k.nx - 1), cy = clampi(si.y, 0, k.ny - 1),
      cz = clampi(si.z, 0, k.nz - 1);
  b.x0 = max(0, cx - k.wx);
  b.x1 = min(k.nx - 1, cx + k.wx);
  b.y0 = max(0, cy - k.wy);
  b.y1 = min(k.ny - 1, cy + k.wy);
  b.l0 = max(0, cz - k.wl);
  b.l1 = min(k.nz - 1, cz + k.wl);
  return b;
}

// Near region of a station: the prisms whose centre lies closer to the
// station than near_q half-diagonals (all of them inside the near box).
// Everything outside the region is at least that far away, so the far-field
// expansion holds there.  In each box column the region's layers are one
// interval; the interval of every (station, box column) is computed once, in
// double, by launch_mesh_near_iv, and every kernel that splits near from far
// pairs reads the same intervals (lo > hi: the column has no near prism).
__device__ __forceinline__ int near_slot(const NearBox& b, int ix, int iy) {
  return (ix - b.x0) + (b.x1 - b.x0 + 1) * (iy - b.y0);
}

// Near region of station s in T (double: the mixed method; float: the FP32
// method), by one warp: Phi once per vertex of the region times the signed
// triple difference of the region's densities around the vertex; lane 0
// writes out[s].
template <typename T>
__device__ __forceinline__ void near_station(const MeshConst& k, const MeshDesc& m, int s,
                                             const double* __restrict__ sxyz,
                                             const int4* __restrict__ si,
                                             const short2* __restrict__ iv,
                                             const int2* __restrict__ lr,
                                             const double* __restrict__ rho,
                                             double* __restrict__ out, int lane,
                                             unsigned* nphi = nullptr) {
  const NearBox b = near_box(si[s], k);
  const int2 L = lr[s];
  if (L.x > L.y) {  // no near prism
    if (lane == 0) out[s] = 0.0;
    return;
  }
  const short2* ivs = iv + (size_t)s * k.nslots;
  const double xs = sxyz[3 * s], ys = sxyz[3 * s + 1], zs = sxyz[3 * s + 2];
  const int nvx = b.x1 - b.x0 + 2, nvy = b.y1 - b.y0 + 2, nvz = L.y - L.x + 2;
  const int nv = nvx * nvy * nvz;
  const long long plane = (long long)m.nx * m.ny;
  T acc = T(0);
  for (int v = lane; v < nv; v += 32) {
    const int a = b.x0 + v % nvx;
    const int bb = b.y0 + (v / nvx) % nvy;
    const int cz = L.x + v / (nvx * nvy);
    // signed triple difference of the region's density around vertex
    // (a, bb, cz): prism ix = a-1 has the vertex as its upper x limit (+),
    // ix = a lower (-); layer l = cz has it as its upper z limit (+), l = cz-1
    // lower (-).
    double D = 0.0;
#pragma unroll
    for (int da = 0; da < 2; da++) {
      const int ix = a - 1 + da;
      if (ix < b.x0 || ix > b.x1) continue;
#pragma unroll
      for (int db = 0; db < 2; db++) {
        const int iy = bb - 1 + db;
        if (iy < b.y0 || iy > b.y1) continue;
        const short2 t = ivs[near_slot(b, ix, iy)];
#pragma unroll
        for (int dc = 0; dc < 2; dc++) {
          const int l = cz - 1 + dc;
          if (l < t.x || l > t.y) continue;
          const double r = rho[ix + (long long)m.nx * iy + plane * l];
          const int neg = (da == 1) ^ (db == 1) ^ (dc == 0);
          D += neg ? -r : r;
        }
      }
    }
    if (D != 0.0) {
      const T x = (T)((m.x0 + a * m.dx) - xs);
      const T y = (T)((m.y0 + bb * m.dy) - ys);
      const T z = (T)((m.zt - cz * m.dz) - zs);
      acc += (T)D * ztm_phi<T>(x, y, z);
      if (nphi) ++*nphi;
    }
  }
  double tot = warp_sum_d((double)acc);
  if (lane == 0) out[s] = tot;
}

// ---- host launchers (prism.cu) ------------------------------------------
MeshConst make_mesh_const(const MeshDesc& m, double near_q);
// Station-relative integer/float decomposition (computed in double once per
// station): x_s - x0 = (ixs + 1/2) dx + ex, likewise y, and
// z_s = z_top - (izs + 1/2) dz + ez, so that station-minus-centre offsets are
// k*d + e with an exact integer k and a small float e (e in units of L0).
void launch_mesh_station_prep(ztm_ctx* c, const MeshDesc& m, double L0, int ns,
                              const double* sxyz, float4* sf, int4* si);
// Column-major float copy of the density: rhoT[c*nzp + l], c = ix + nx*iy,
// padded layers zero.  nmodels > 1: model-major blocks of ncols*nzp floats.
void launch_mesh_transpose(ztm_ctx* c, const MeshConst& k, int nmodels, const double* rho,
                           float* rhoT);
// Near-region intervals: iv[s*nslots + slot] (layers lo..hi) and the
// station's overall layer range lr[s] = (lmin, lmax) (lmin > lmax: none).
void launch_mesh_near_iv(ztm_ctx* c, const MeshConst& k, const MeshDesc& m, int ns,
                         const int4* si, const double* sxyz, short2* iv, int2* lr);
