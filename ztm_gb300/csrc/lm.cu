// lm.cu - the damped Gauss-Newton step of ZTM's optimiser on the GPU.
//
// LMA::fit (TFM.cpp:155-167) forms, per iteration, JJ = MTM(J) = J^T J
// (zmath.cpp:260-262, one host thread per column), M = diag(diag(JJ)),
// A = diag(1/sig^2), and for every damping pair d of its grid the trial
// B = b + inv(JJ + d0 M + d1 A) J^T r (TFM.cpp:160), the inverse by
// Gauss-Jordan elimination with partial pivoting (zmath.cpp:129-140), one
// host thread per damping pair.  Here:
//   lm_jtj_kernel   J^T J in double, 64 x 64 output tiles (16 x 16 threads,
//                   4 x 4 outputs each) over 16-row slabs of J staged in
//                   shared memory; tiles on and above the diagonal, mirrored;
//   lm_jtr_kernel   J^T r, thread per parameter (coalesced over J's rows);
//   lm_assemble     one augmented system [JJ + d0 M + d1 A | J^T r] per
//                   damping pair;
//   lm_panel /      blocked LU with partial pivoting of the augmented
//   lm_trsm /       systems, all pairs at once, and back substitution (see
//   lm_update /     below); the right-hand column becomes the step;
//   lm_backsolve
//   lm_finish       B = b + step (b where the system was singular, as the
//                   reference's inv returns zeros there).
// The reference inverts by Gauss-Jordan and then multiplies by J^T and r;
// factorising with the right-hand side attached gives the same step up to
// rounding, with the same pivots, in two thirds of the multiply-adds and with
// most of them in compute-bound tiles (Gauss-Jordan on all four 2700-column
// systems re-read the 233 MB of them from DRAM once per column).  Double
// throughout (the normal equations square the condition number).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "ztm_internal.cuh"

namespace {

constexpr int LM_T = 64;  // output tile edge
constexpr int LM_K = 16;  // rows of J per shared-memory slab

// JJ[i][j] = sum_r J[r][i] J[r][j] for the tiles (bi <= bj), written to both
// halves.  J is nrows x ncols, row-major.
__global__ void __launch_bounds__(256)
    lm_jtj_kernel(const double* __restrict__ J, int nrows, int ncols, double* __restrict__ JJ) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bi > bj) return;
  __shared__ double As[LM_K][LM_T + 1], Bs[LM_K][LM_T + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = bi * LM_T, j0 = bj * LM_T;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  for (int r0 = 0; r0 < nrows; r0 += LM_K) {
    __syncthreads();
    for (int q = threadIdx.x; q < LM_K * LM_T; q += 256) {
      const int rr = q / LM_T, cc = q % LM_T, r = r0 + rr;
      As[rr][cc] = (r < nrows && i0 + cc < ncols) ? J[(long long)r * ncols + i0 + cc] : 0.0;
      Bs[rr][cc] = (r < nrows && j0 + cc < ncols) ? J[(long long)r * ncols + j0 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < LM_K; k++) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        a[q] = As[k][ty + 16 * q];
        b[q] = Bs[k][tx + 16 * q];
      }
#pragma unroll
      for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
  }
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
      if (i < ncols && j < ncols) {
        JJ[(long long)i * ncols + j] = acc[p][q];
        JJ[(long long)j * ncols + i] = acc[p][q];
      }
    }
}

__global__ void lm_jtr_kernel(const double* __restrict__ J, int nrows, int ncols,
                              const double* __restrict__ r, double* __restrict__ g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncols) return;
  double s = 0.0;
  for (int k = 0; k < nrows; k++) s = fma(J[(long long)k * ncols + i], r[k], s);
  g[i] = s;
}

// aug[d] = [JJ + d0 diag(JJ) + d1 diag(1/sig^2) | g], row stride n + 1.
__global__ void lm_assemble(int n, int nd, const double* __restrict__ JJ,
                            const double* __restrict__ g, const double* __restrict__ sig,
                            const double* __restrict__ dm, double* __restrict__ aug) {
  const long long w = n + 1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)nd * n * w) return;
  const int d = (int)(t / (n * w));
  const long long e = t - (long long)d * n * w;
  const int i = (int)(e / w), j = (int)(e % w);
  double v;
  if (j == n) {
    v = g[i];
  } else {
    v = JJ[(long long)i * n + j];
    if (i == j) v = (v + dm[2 * d] * v) + dm[2 * d + 1] * (1.0 / (sig[i] * sig[i]));
  }
  aug[t] = v;
}

// ---- the damped systems by blocked LU ---------------------------------------
// Right-looking LU with partial pivoting of the augmented matrix [A | g]
// (row stride n + 1), LM_NB columns per panel, every damping pair at once:
//   lm_panel     one block per pair: per column of the panel the first row at
//                or below the diagonal with the largest |a| (the reference's
//                pivot rule, zmath.cpp:132; the rows below the diagonal see the
//                same updates in Gauss-Jordan elimination, so the pivots are
//                the same), the swap of the two rows from the panel's first
//                column on, the multipliers a[r][c] /= a[c][c], and the update of
//                the panel's remaining columns; a zero pivot marks the pair
//                singular;
//   lm_trsm      the panel rows of the trailing columns (the right-hand side
//                included): U12 = L11^-1 A12, a thread per column;
//   lm_update    A22 -= L21 U12 in 64 x 64 tiles, the panel's LM_NB columns of
//                L21 and rows of U12 staged in shared memory;
//   lm_backsolve one block per pair: U x = y from the last row up.
// The right-hand side column ends as the step.
constexpr int LM_NB = 8;
constexpr int LM_SMEM_ROWS = 3500;  // panels of up to this many rows in shared memory

// The panel in shared memory (rows k0 .. n-1, LM_NB doubles each, 219 KB at
// most): the same steps as lm_panel without a trip to L2 per step, the
// pivot rows recorded in piv (global indices) for lm_trsm to apply to the
// columns right of the panel.
__global__ void __launch_bounds__(1024)
    lm_panel_smem(int n, int k0, int nb, double* __restrict__ aug, int* __restrict__ piv,
                  int* __restrict__ singular) {
  extern __shared__ double P[];  // [n - k0][LM_NB]
  const int d = blockIdx.x;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  const int R = n - k0;
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  __shared__ int s_p;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int t = threadIdx.x; t < R * LM_NB; t += blockDim.x) {
    const int r = t / LM_NB, m = t % LM_NB;
    P[t] = m < nb ? a[(long long)(k0 + r) * w + k0 + m] : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < nb; c++) {
    double best = -1.0;
    int bi = R;
    for (int r = c + threadIdx.x; r < R; r += blockDim.x) {
      const double v = fabs(P[r * LM_NB + c]);
      if (v > best) {
        best = v;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_down_sync(0xffffffffu, best, o);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
      if (v2 > best || (v2 == best && i2 < bi)) {
        best = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      s_v[warp] = best;
      s_i[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bv = s_v[0];
      int bp = s_i[0];
      for (int q = 1; q < nw; q++)
        if (s_v[q] > bv || (s_v[q] == bv && s_i[q] < bp)) {
          bv = s_v[q];
          bp = s_i[q];
        }
      s_p = (bv > 0.0) ? bp : -1;
      if (bv <= 0.0) singular[d] = 1;
      else piv[(long long)d * n + k0 + c] = k0 + bp;
    }
    __syncthreads();
    const int p = s_p;
    if (p < 0) return;
    if (p != c && threadIdx.x < LM_NB) {
      const double x = P[c * LM_NB + threadIdx.x];
      P[c * LM_NB + threadIdx.x] = P[p * LM_NB + threadIdx.x];
      P[p * LM_NB + threadIdx.x] = x;
    }
    __syncthreads();
    const double finv = 1.0 / P[c * LM_NB + c];
    for (int r = c + 1 + threadIdx.x; r < R; r += blockDim.x) {
      double* row = P + r * LM_NB;
      const double l = row[c] * finv;
      row[c] = l;
#pragma unroll
      for (int j = 0; j < LM_NB; j++)
        if (j > c && j < nb) row[j] = fma(-l, P[c * LM_NB + j], row[j]);
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < R * LM_NB; t += blockDim.x) {
    const int r = t / LM_NB, m = t % LM_NB;
    if (m < nb) a[(long long)(k0 + r) * w + k0 + m] = P[t];
  }
}

__global__ void __launch_bounds__(1024)
    lm_panel(int n, int k0, int nb, double* __restrict__ aug, int* __restrict__ singular) {
  const int d = blockIdx.x;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  __shared__ int s_p;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = k0; c < k0 + nb; c++) {
    double best = -1.0;
    int bi = n;
    for (int r = c + threadIdx.x; r < n; r += blockDim.x) {
      const double v = fabs(a[r * w + c]);
      if (v > best) {  // rows visited in increasing order: ties keep the first
        best = v;
        bi = r;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_down_sync(0xffffffffu, best, o);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
      if (v2 > best || (v2 == best && i2 < bi)) {
        best = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      s_v[warp] = best;
      s_i[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bv = s_v[0];
      int bp = s_i[0];
      for (int q = 1; q < nw; q++)
        if (s_v[q] > bv || (s_v[q] == bv && s_i[q] < bp)) {
          bv = s_v[q];
          bp = s_i[q];
        }
      s_p = (bv > 0.0) ? bp : -1;
      if (bv <= 0.0) singular[d] = 1;
    }
    __syncthreads();
    const int p = s_p;
    if (p < 0) return;  // every thread read the same verdict
    if (p != c)  // from the panel's first column: its multipliers move with the rows
      for (int j = k0 + threadIdx.x; j <= n; j += blockDim.x) {
        const double x = a[(long long)c * w + j];
        a[(long long)c * w + j] = a[(long long)p * w + j];
        a[(long long)p * w + j] = x;
      }
    __syncthreads();
    const double finv = 1.0 / a[(long long)c * w + c];
    for (int r = c + 1 + threadIdx.x; r < n; r += blockDim.x) a[r * w + c] *= finv;
    __syncthreads();
    // the panel's columns right of c (fewer than LM_NB): 16 columns x 64 rows
    // per pass, a row's columns on neighbouring threads
    const int j = c + 1 + (threadIdx.x & (LM_NB - 1));
    if (j < k0 + nb) {
      const double u = a[(long long)c * w + j];
      for (int r = c + 1 + (threadIdx.x >> 4); r < n; r += blockDim.x >> 4)
        a[r * w + j] = fma(-a[r * w + c], u, a[r * w + j]);
    }
    __syncthreads();
  }
}

// U12 = L11^-1 A12 for the panel rows k0 .. k0+nb-1 and the columns right of
// the panel (the right-hand side included), a thread per column.
__global__ void __launch_bounds__(256)
    lm_trsm(int n, int k0, int nb, double* __restrict__ aug, const int* __restrict__ piv,
            const int* __restrict__ singular) {
  const int d = blockIdx.y;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  __shared__ double L[LM_NB][LM_NB];
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int i = t / nb, m = t % nb;
    L[i][m] = a[(long long)(k0 + i) * w + k0 + m];
  }
  __syncthreads();
  const int j = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (j > n) return;
  if (piv)  // the panel's row swaps, in order, on this column
    for (int i = 0; i < nb; i++) {
      const int p = piv[(long long)d * n + k0 + i];
      if (p != k0 + i) {
        const double t = a[(long long)(k0 + i) * w + j];
        a[(long long)(k0 + i) * w + j] = a[(long long)p * w + j];
        a[(long long)p * w + j] = t;
      }
    }
  double x[LM_NB];
#pragma unroll
  for (int i = 0; i < LM_NB; i++) x[i] = i < nb ? a[(long long)(k0 + i) * w + j] : 0.0;
#pragma unroll
  for (int i = 1; i < LM_NB; i++)
#pragma unroll
    for (int m = 0; m < i; m++) x[i] = fma(-L[i][m], x[m], x[i]);
#pragma unroll
  for (int i = 0; i < LM_NB; i++)
    if (i < nb) a[(long long)(k0 + i) * w + j] = x[i];
}

// A22 -= L21 U12: rows k0+nb .. n-1, columns k0+nb .. n; 64 x 64 tiles, 16 x 16
// threads with 4 x 4 outputs each.
__global__ void __launch_bounds__(256)
    lm_update(int n, int k0, int nb, double* __restrict__ aug, const int* __restrict__ singular) {
  const int d = blockIdx.z;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  __shared__ double Ls[LM_T][LM_NB + 1], Us[LM_NB][LM_T + 1];
  const int r0 = k0 + nb + blockIdx.y * LM_T, j0 = k0 + nb + blockIdx.x * LM_T;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int q = threadIdx.x; q < LM_T * LM_NB; q += 256) {
    const int rr = q / LM_NB, m = q % LM_NB, r = r0 + rr;
    Ls[rr][m] = (r < n && m < nb) ? a[(long long)r * w + k0 + m] : 0.0;
    const int mm = q / LM_T, cc = q % LM_T, j = j0 + cc;
    Us[mm][cc] = (j <= n && mm < nb) ? a[(long long)(k0 + mm) * w + j] : 0.0;
  }
  __syncthreads();
  double acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[p][q] = 0.0;
#pragma unroll
  for (int m = 0; m < LM_NB; m++) {
    double l[4], u[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      l[q] = Ls[ty + 16 * q][m];
      u[q] = Us[m][tx + 16 * q];
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[p][q] = fma(l[p], u[q], acc[p][q]);
  }
#pragma unroll
  for (int p = 0; p < 4; p++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = r0 + ty + 16 * p, j = j0 + tx + 16 * q;
      if (r < n && j <= n) a[(long long)r * w + j] -= acc[p][q];
    }
}

// U x = y (y the right-hand side column, overwritten by x), one block per
// pair, 32 rows at a time from the bottom: warp 0 solves the block's
// triangle (lane l holds row l's right-hand side), then every thread updates
// the right-hand sides of the rows above with the block's 32 unknowns.
__global__ void __launch_bounds__(1024)
    lm_backsolve(int n, double* __restrict__ aug, const int* __restrict__ singular) {
  const int d = blockIdx.x;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  __shared__ double s_x[32];
  const int lane = threadIdx.x & 31;
  for (int b0 = ((n - 1) / 32) * 32; b0 >= 0; b0 -= 32) {
    const int be = min(n, b0 + 32);
    if (threadIdx.x < 32) {
      const int row = b0 + lane;
      double y = row < be ? a[(long long)row * w + n] : 0.0;
      for (int i = be - 1; i >= b0; i--) {
        const double xi = __shfl_sync(0xffffffffu, y, i - b0) / a[(long long)i * w + i];
        if (lane < i - b0) y = fma(-a[(long long)row * w + i], xi, y);
        if (lane == i - b0) y = xi;
      }
      if (row < be) {
        a[(long long)row * w + n] = y;
        s_x[lane] = y;
      }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < b0; r += blockDim.x) {
      double acc = 0.0;
      for (int i = b0; i < be; i++) acc = fma(a[(long long)r * w + i], s_x[i - b0], acc);
      a[(long long)r * w + n] -= acc;
    }
    __syncthreads();
  }
}

__global__ void lm_finish(int n, int nd, const double* __restrict__ aug,
                          const int* __restrict__ singular, const double* __restrict__ b,
                          double* __restrict__ B) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)nd * n) return;
  const int d = (int)(t / n), i = (int)(t % n);
  const double step = singular[d] ? 0.0 : aug[(long long)d * n * (n + 1) + (long long)i * (n + 1) + n];
  B[t] = b[i] + step;
}

}  // namespace

extern "C" int ztm_lm_steps(ztm_ctx* c, const double* J, int nrows, int ncols, const double* r,
                            const double* b, const double* sig, const double* damping, int nd,
                            double* B, double* JJ, int flags) {
  if (!c) return ZTM_ERR_ARG;
  c->err.clear();
  if (!J || !r || !b || !sig || !damping || !B) return ztm_fail(c, ZTM_ERR_ARG, "null argument");
  if (nrows < 1 || ncols < 1 || nd < 1) return ztm_fail(c, ZTM_ERR_ARG, "sizes must be >= 1");
  if (flags & ~ZTM_FLAG_DEVICE_PTRS) return ztm_fail(c, ZTM_ERR_ARG, "unknown flag");
  if (ncols > 32768 || (long long)nd * ncols * (ncols + 1) > (1LL << 31))
    return ztm_fail(c, ZTM_ERR_RANGE, "normal equations too large (ncols <= 32768, nd*ncols^2 < 2^31)");
  const bool dev = (flags & ZTM_FLAG_DEVICE_PTRS) != 0;
  const size_t n = ncols, m = nrows;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device && cudaSetDevice(c->device) != cudaSuccess)
    return ztm_fail(c, ZTM_ERR_NODEV, "cannot select device");
  struct Restore {
    int p, d;
    ~Restore() {
      if (p >= 0 && p != d) cudaSetDevice(p);
    }
  } restore{prev, c->device};
  const size_t need = WsCarver::need(m * n * 8) + 3 * WsCarver::need(m * 8 + n * 8) +
                      WsCarver::need(n * n * 8) + WsCarver::need((size_t)nd * 16) +
                      WsCarver::need((size_t)nd * n * (n + 1) * 8) + WsCarver::need((size_t)nd * 4) +
                      WsCarver::need((size_t)nd * n * 4) +
                      WsCarver::need((size_t)nd * n * 8) + 4096;
  int rc = ztm_ws_reserve(c, need);
  if (rc) return rc;
  WsCarver wc(c->ws);
  double* s_J = wc.take<double>(m * n);
  double* s_r = wc.take<double>(m);
  double* s_b = wc.take<double>(n);
  double* s_sig = wc.take<double>(n);
  double* s_JJ = wc.take<double>(n * n);
  double* s_dm = wc.take<double>((size_t)nd * 2);
  double* aug = wc.take<double>((size_t)nd * n * (n + 1));
  int* singular = wc.take<int>((size_t)nd);
  int* piv = wc.take<int>((size_t)nd * n);
  double* s_B = wc.take<double>((size_t)nd * n);
  double* g = wc.take<double>(n);
  const void *pJ, *pr, *pb, *ps, *pd;
  if ((rc = ztm_stage_in(c, J, m * n * 8, dev, s_J, &pJ))) return rc;
  if ((rc = ztm_stage_in(c, r, m * 8, dev, s_r, &pr))) return rc;
  if ((rc = ztm_stage_in(c, b, n * 8, dev, s_b, &pb))) return rc;
  if ((rc = ztm_stage_in(c, sig, n * 8, dev, s_sig, &ps))) return rc;
  if ((rc = ztm_stage_in(c, damping, (size_t)nd * 16, dev, s_dm, &pd))) return rc;
  double* oJJ = (dev && JJ) ? JJ : s_JJ;
  double* oB = dev ? B : s_B;
  cudaMemsetAsync(singular, 0, (size_t)nd * 4, c->stream);
  const int tiles = (int)((n + LM_T - 1) / LM_T);
  {
    ZtmProf prof_(c, "lm");
    lm_jtj_kernel<<<dim3(tiles, tiles), 256, 0, c->stream>>>((const double*)pJ, nrows, ncols, oJJ);
    lm_jtr_kernel<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>((const double*)pJ, nrows,
                                                                       ncols, (const double*)pr, g);
    const long long tot = (long long)nd * n * (n + 1);
    lm_assemble<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(
        ncols, nd, oJJ, g, (const double*)ps, (const double*)pd, aug);
    const bool smem_panel = ncols <= LM_SMEM_ROWS;
    if (smem_panel)
      cudaFuncSetAttribute(lm_panel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)((size_t)ncols * LM_NB * 8));
    for (int k0 = 0; k0 < ncols; k0 += LM_NB) {
      const int nb = std::min(LM_NB, ncols - k0);
      if (smem_panel)
        lm_panel_smem<<<nd, 1024, (size_t)(ncols - k0) * LM_NB * 8, c->stream>>>(ncols, k0, nb, aug,
                                                                                piv, singular);
      else
        lm_panel<<<nd, 1024, 0, c->stream>>>(ncols, k0, nb, aug, singular);
      const int rest = ncols + 1 - (k0 + nb);  // columns right of the panel, RHS included
      lm_trsm<<<dim3((unsigned)((rest + 255) / 256), nd), 256, 0, c->stream>>>(
          ncols, k0, nb, aug, smem_panel ? piv : nullptr, singular);
      const int rows = ncols - (k0 + nb);
      if (rows > 0)
        lm_update<<<dim3((unsigned)((rest + LM_T - 1) / LM_T), (unsigned)((rows + LM_T - 1) / LM_T),
                         nd),
                    256, 0, c->stream>>>(ncols, k0, nb, aug, singular);
    }
    lm_backsolve<<<nd, 1024, 0, c->stream>>>(ncols, aug, singular);
    lm_finish<<<(unsigned)(((size_t)nd * n + 255) / 256), 256, 0, c->stream>>>(
        ncols, nd, aug, singular, (const double*)pb, oB);
  }
  c->launches += 5 + 3LL * ((ncols + LM_NB - 1) / LM_NB);
  if ((rc = ztm_after_launch(c, "normal equations"))) return rc;
  if (!dev) {
    if (JJ) cudaMemcpyAsync(JJ, oJJ, n * n * 8, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(B, oB, (size_t)nd * n * 8, cudaMemcpyDeviceToHost, c->stream);
  }
  return ztm_finish(c, dev, nullptr, nullptr, 0, "normal equations");
}
