// mesh_far.cuh - the far field of one model on a 3-D prism mesh, float, for
// a thread's station against the columns of a shared-memory stage: the
// column loop of the mixed forward (prism.cu, far_kernel) and of the batched
// forward's one-model jobs (batch.cu).  Density of a column: nzp floats,
// layer l at l, zero in the padding layers l >= nz.  Near-region layers
// [elo, elo + espan] of a column in the station's near box come from the
// interval table ivs[station][box column] (launch_mesh_near_iv).
#pragma once
#include <cuda_runtime.h>

#include "prism_common.cuh"
#include "ztm_internal.cuh"

#ifdef __CUDACC__

namespace meshfar {

// Per-thread station state of the far kernel for one tile of stations.
struct FarStation {
  float ex, ey, ez;
  int ixs, iys, izs;
  NearBox nb;
};

// Eight layers l0..l0+7 of one column: adds rho * (far value) to g (two
// lanes: even and odd layers).  T2: the second-order form for the whole warp.
// MASK: drop the layers of the station's near region [elo, elo + espan] and
// the padding layers >= nz (select, not multiply: a NaN there is dropped).
template <bool T2, bool MASK>
__device__ __forceinline__ float2 far_group(const float* col, int l0, float fl,
                                            const float2 (&Zb)[4], float2 zstep,
                                            const ColPoly2& cp2, float2 c2t, int elo,
                                            unsigned espan, int nz, float2 g) {
  const float4 ra = *reinterpret_cast<const float4*>(col + l0);
  const float4 rb = *reinterpret_cast<const float4*>(col + l0 + 4);
  const float2 l2 = make_float2(fl, fl);  // fl = l0, carried in float (no conversion)
  float2 v[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float2 Z = __ffma2_rn(l2, zstep, Zb[j]);  // Z(l) = (l - izs) dz + ez
    v[j] = T2 ? far_unit2_t2(Z, cp2, c2t) : far_unit2(Z, cp2);
  }
  if (MASK) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int la = l0 + 2 * j, lb = la + 1;
      if (((unsigned)(la - elo) <= espan) || la >= nz) v[j].x = 0.f;
      if (((unsigned)(lb - elo) <= espan) || lb >= nz) v[j].y = 0.f;
    }
  }
  g = __ffma2_rn(make_float2(ra.x, ra.y), v[0], g);
  g = __ffma2_rn(make_float2(ra.z, ra.w), v[1], g);
  g = __ffma2_rn(make_float2(rb.x, rb.y), v[2], g);
  return __ffma2_rn(make_float2(rb.z, rb.w), v[3], g);
}

// All layers of one column: groups [0, lmask) with the near mask, full
// groups up to nz8 without, a masked tail group if nz is not a multiple of 8.
// Plain float sums over 32 layers (two lanes of 16), compensated across.
template <bool T2>
__device__ __forceinline__ void far_column(const float* col, int lmask, int nz8, int nz,
                                           const float2 (&Zb)[4], float2 zstep,
                                           const ColPoly2& cp2, float2 c2t, int elo,
                                           unsigned espan, Kahan& acc) {
  float2 g = make_float2(0.f, 0.f);
  int l0 = 0;
  float fl = 0.f;
  for (; l0 < lmask; l0 += 8, fl += 8.f) {
    g = far_group<T2, true>(col, l0, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    if ((l0 & 24) == 24) {
      acc.add(g.x + g.y);
      g = make_float2(0.f, 0.f);
    }
  }
  // unmasked groups: singly up to a 32-layer boundary, then eight at a time
  // over whole 64-layer blocks and four at a time over a 32-layer block (one
  // loop test per block, one compensation per 32 layers), singly after
  for (; l0 < nz8 && (l0 & 31); l0 += 8, fl += 8.f) {
    g = far_group<T2, false>(col, l0, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    if ((l0 & 24) == 24) {
      acc.add(g.x + g.y);
      g = make_float2(0.f, 0.f);
    }
  }
  for (; l0 + 64 <= nz8; l0 += 64, fl += 64.f) {
    g = far_group<T2, false>(col, l0, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 8, fl + 8.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 16, fl + 16.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 24, fl + 24.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    acc.add(g.x + g.y);
    g = far_group<T2, false>(col, l0 + 32, fl + 32.f, Zb, zstep, cp2, c2t, elo, espan, nz,
                             make_float2(0.f, 0.f));
    g = far_group<T2, false>(col, l0 + 40, fl + 40.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 48, fl + 48.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 56, fl + 56.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    acc.add(g.x + g.y);
    g = make_float2(0.f, 0.f);
  }
  for (; l0 + 32 <= nz8; l0 += 32, fl += 32.f) {
    g = far_group<T2, false>(col, l0, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 8, fl + 8.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 16, fl + 16.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    g = far_group<T2, false>(col, l0 + 24, fl + 24.f, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    acc.add(g.x + g.y);
    g = make_float2(0.f, 0.f);
  }
  for (; l0 < nz8; l0 += 8, fl += 8.f) {
    g = far_group<T2, false>(col, l0, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
    if ((l0 & 24) == 24) {
      acc.add(g.x + g.y);
      g = make_float2(0.f, 0.f);
    }
  }
  if (nz8 < nz) g = far_group<T2, true>(col, nz8, fl, Zb, zstep, cp2, c2t, elo, espan, nz, g);
  acc.add(g.x + g.y);
}

// Two columns A and B, eight layers l0..l0+7, second-order form, no mask:
// one Z per layer pair serves both columns.
__device__ __forceinline__ float2 far_group_pair(const float* colA, const float* colB, int l0,
                                                 float fl, const float2 (&Zb)[4], float2 zstep,
                                                 const ColPoly2& cpA, float2 c2tA,
                                                 const ColPoly2& cpB, float2 c2tB, float2 g) {
  const float4 raA = *reinterpret_cast<const float4*>(colA + l0);
  const float4 rbA = *reinterpret_cast<const float4*>(colA + l0 + 4);
  const float4 raB = *reinterpret_cast<const float4*>(colB + l0);
  const float4 rbB = *reinterpret_cast<const float4*>(colB + l0 + 4);
  const float2 l2 = make_float2(fl, fl);
  float2 vA[4], vB[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float2 Z = __ffma2_rn(l2, zstep, Zb[j]);
    vA[j] = far_unit2_t2(Z, cpA, c2tA);
    vB[j] = far_unit2_t2(Z, cpB, c2tB);
  }
  g = __ffma2_rn(make_float2(raA.x, raA.y), vA[0], g);
  g = __ffma2_rn(make_float2(raB.x, raB.y), vB[0], g);
  g = __ffma2_rn(make_float2(raA.z, raA.w), vA[1], g);
  g = __ffma2_rn(make_float2(raB.z, raB.w), vB[1], g);
  g = __ffma2_rn(make_float2(rbA.x, rbA.y), vA[2], g);
  g = __ffma2_rn(make_float2(rbB.x, rbB.y), vB[2], g);
  g = __ffma2_rn(make_float2(rbA.z, rbA.w), vA[3], g);
  return __ffma2_rn(make_float2(rbB.z, rbB.w), vB[3], g);
}

// Layers 0 .. nl - 1 of two columns (nl a multiple of 8: nz, or the padded
// nzp where the padding layers' K is finite): plain float sums over 16
// layers of both (32 terms), compensated across.
__device__ __forceinline__ void far_column_pair(const float* colA, const float* colB, int nl,
                                                const float2 (&Zb)[4], float2 zstep,
                                                const ColPoly2& cpA, float2 c2tA,
                                                const ColPoly2& cpB, float2 c2tB, Kahan& acc) {
  int l0 = 0;
  float fl = 0.f;
  const float2 z0 = make_float2(0.f, 0.f);
  for (; l0 + 64 <= nl; l0 += 64, fl += 64.f) {
#pragma unroll
    for (int h = 0; h < 4; h++) {
      float2 g = far_group_pair(colA, colB, l0 + 16 * h, fl + 16.f * h, Zb, zstep, cpA, c2tA,
                                cpB, c2tB, z0);
      g = far_group_pair(colA, colB, l0 + 16 * h + 8, fl + 16.f * h + 8.f, Zb, zstep, cpA, c2tA,
                         cpB, c2tB, g);
      acc.add(g.x + g.y);
    }
  }
  for (; l0 + 16 <= nl; l0 += 16, fl += 16.f) {
    float2 g = far_group_pair(colA, colB, l0, fl, Zb, zstep, cpA, c2tA, cpB, c2tB, z0);
    g = far_group_pair(colA, colB, l0 + 8, fl + 8.f, Zb, zstep, cpA, c2tA, cpB, c2tB, g);
    acc.add(g.x + g.y);
  }
  if (l0 < nl) {
    const float2 g = far_group_pair(colA, colB, l0, fl, Zb, zstep, cpA, c2tA, cpB, c2tB, z0);
    acc.add(g.x + g.y);
  }
}

// One shared-memory stage (ncol columns starting at column cs) against this
// thread's station; adds to acc.  Every lane runs the loop (inactive lanes
// on dummy data) for the warp votes.
// COUNT: add the (station, prism) slots this thread evaluates to cnt by
// form: [0] sixth order, [1] second order, [2] second order by column pairs.
template <bool COUNT>
__device__ __forceinline__ void far_stage(const short2* __restrict__ ivs, const MeshConst& k,
                                          const FarCoef& fc, const FarStation& t, int s, int Lm,
                                          const float* rs, int cs, int ncol, Kahan& acc,
                                          unsigned (&cnt)[3]) {
  const float2 zstep = make_float2(k.dzn, k.dzn);
  // Z of layers 2j, 2j+1 of a group at l0 = 0; a group at l0 adds l0 dz
  float2 Zb[4];
#pragma unroll
  for (int j = 0; j < 4; j++)
    Zb[j] = make_float2(fmaf((float)(2 * j - t.izs), k.dzn, t.ez),
                        fmaf((float)(2 * j + 1 - t.izs), k.dzn, t.ez));
  const int nz8 = k.nz & ~7;
  const int lm8 = min((Lm + 7) & ~7, nz8);
  // column pairs run over all nzp layers unmasked: where nz is not a
  // multiple of 8 that needs every lane's station above the mesh bottom
  // (izs < nz), whose Z at a padding layer is then at least half a layer, so
  // that K there is finite and the zero density adds nothing
  const bool pairs = nz8 == k.nz || __all_sync(0xffffffffu, t.izs < k.nz);
  int ix = cs % k.nx, iy = cs / k.nx;
  for (int q = 0; q < ncol; q++) {
    // two unmasked second-order columns at once where the warp allows it
    if (pairs && q + 1 < ncol) {
      int ix1 = ix + 1, iy1 = iy;
      if (ix1 == k.nx) {
        ix1 = 0;
        ++iy1;
      }
      const float XA = fmaf((float)(t.ixs - ix), k.dxn, t.ex);
      const float YA = fmaf((float)(t.iys - iy), k.dyn, t.ey);
      const float XB = fmaf((float)(t.ixs - ix1), k.dxn, t.ex);
      const float YB = fmaf((float)(t.iys - iy1), k.dyn, t.ey);
      const float XA2 = XA * XA, YA2 = YA * YA, rhA = XA2 + YA2;
      const float XB2 = XB * XB, YB2 = YB * YB, rhB = XB2 + YB2;
      const bool nclA = ix >= t.nb.x0 && ix <= t.nb.x1 && iy >= t.nb.y0 && iy <= t.nb.y1;
      const bool nclB = ix1 >= t.nb.x0 && ix1 <= t.nb.x1 && iy1 >= t.nb.y0 && iy1 <= t.nb.y1;
      const bool unmasked = lm8 == 0 || !__any_sync(0xffffffffu, nclA || nclB);
      if (unmasked && __all_sync(0xffffffffu, fminf(rhA, rhB) >= k.rh_t2)) {
        const float cA = fmaf(-fc.a1, rhA, fmaf(XA2, fc.cA, YA2 * fc.cB));
        const float cB = fmaf(-fc.a1, rhB, fmaf(XB2, fc.cA, YB2 * fc.cB));
        ColPoly2 cpA, cpB;
        cpA.rh = make_float2(rhA, rhA);
        cpB.rh = make_float2(rhB, rhB);
        cpA.a1 = cpB.a1 = make_float2(fc.a1, fc.a1);
        cpA.C2 = cpA.C3 = cpA.C4 = cpA.C5 = cpA.C6 = make_float2(0.f, 0.f);
        cpB.C2 = cpB.C3 = cpB.C4 = cpB.C5 = cpB.C6 = make_float2(0.f, 0.f);
        far_column_pair(rs + q * k.nzp, rs + (q + 1) * k.nzp, k.nzp, Zb, zstep, cpA,
                        make_float2(cA, cA), cpB, make_float2(cB, cB), acc);
        if (COUNT) cnt[2] += 2 * k.nzp;
        q++;
        ix = ix1 + 1;
        iy = iy1;
        if (ix == k.nx) {
          ix = 0;
          ++iy;
        }
        continue;
      }
    }
    const float X = fmaf((float)(t.ixs - ix), k.dxn, t.ex);
    const float Y = fmaf((float)(t.iys - iy), k.dyn, t.ey);
    const float X2 = X * X, Y2 = Y * Y, rh = X2 + Y2;
    const bool ncl = ix >= t.nb.x0 && ix <= t.nb.x1 && iy >= t.nb.y0 && iy <= t.nb.y1;
    int elo = k.nz;
    unsigned espan = 0u;
    if (ncl) {  // the column's near-region layers
      const short2 iv = ivs[(size_t)s * k.nslots + near_slot(t.nb, ix, iy)];
      if (iv.x <= iv.y) {
        elo = iv.x;
        espan = (unsigned)(iv.y - iv.x);
      }
    }
    const float* col = rs + q * k.nzp;
    // a column lies in some lane's near box only near the warp's stations:
    // test that once per column for the whole warp
    const int lmask = __any_sync(0xffffffffu, ncl) ? lm8 : 0;
    // every lane of the warp far enough for the second-order form, which
    // needs only C2t = a0 - a1 rh of the column polynomial
    if (__all_sync(0xffffffffu, rh >= k.rh_t2)) {
      const float c2t = fmaf(-fc.a1, rh, fmaf(X2, fc.cA, Y2 * fc.cB));
      ColPoly2 cp2;
      cp2.rh = make_float2(rh, rh);
      cp2.a1 = make_float2(fc.a1, fc.a1);
      cp2.C2 = cp2.C3 = cp2.C4 = cp2.C5 = cp2.C6 = make_float2(0.f, 0.f);  // unused by the form
      far_column<true>(col, lmask, nz8, k.nz, Zb, zstep, cp2, make_float2(c2t, c2t), elo, espan,
                       acc);
      if (COUNT) cnt[1] += k.nzp;
    } else {
      const ColPoly2 cp2 = col_poly2(col_poly(X, Y, fc), fc.a1);
      far_column<false>(col, lmask, nz8, k.nz, Zb, zstep, cp2, make_float2(0.f, 0.f), elo, espan,
                        acc);
      if (COUNT) cnt[0] += k.nzp;
    }
    if (++ix == k.nx) {
      ix = 0;
      ++iy;
    }
  }
}

}  // namespace meshfar

#endif  // __CUDACC__
