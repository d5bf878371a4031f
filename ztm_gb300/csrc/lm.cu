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
//   lm_pivot /      Gauss-Jordan with partial pivoting on all pairs at once
//   lm_eliminate    (grid.z = pair): per column the first largest |a| at or
//                   below the diagonal (the reference's pivot rule), the row
//                   swap and the division of the pivot row, then every other
//                   row's elimination; the right-hand column becomes the step;
//   lm_finish       B = b + step (b where the system was singular, as the
//                   reference's inv returns zeros there).
// The reference inverts and then multiplies by J^T and r; eliminating on the
// right-hand side gives the same step up to rounding.  Double throughout (the
// normal equations square the condition number).
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

// Column c of pair d (one block per pair): the first row at or below c with
// the largest |a| (the reference's pivot rule, zmath.cpp:132), the swap, and
// the division of the pivot row by its diagonal; a zero pivot marks the pair
// singular.
__global__ void __launch_bounds__(256)
    lm_pivot(int n, int c, double* __restrict__ aug, int* __restrict__ singular) {
  const int d = blockIdx.x;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  __shared__ double s_v[256];
  __shared__ int s_i[256];
  double best = -1.0;
  int bi = n;
  for (int r = c + threadIdx.x; r < n; r += 256) {
    const double v = fabs(a[r * w + c]);
    if (v > best) {  // rows visited in increasing order: ties keep the first
      best = v;
      bi = r;
    }
  }
  s_v[threadIdx.x] = best;
  s_i[threadIdx.x] = bi;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double v2 = s_v[threadIdx.x + o];
      const int i2 = s_i[threadIdx.x + o];
      if (v2 > s_v[threadIdx.x] || (v2 == s_v[threadIdx.x] && i2 < s_i[threadIdx.x])) {
        s_v[threadIdx.x] = v2;
        s_i[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  const int im = s_i[0];
  __shared__ double s_f;
  if (threadIdx.x == 0) s_f = im < n ? a[(long long)im * w + c] : 0.0;
  __syncthreads();  // the pivot is read before any thread writes the rows
  const double f = s_f;
  if (f == 0.0) {
    if (threadIdx.x == 0) singular[d] = 1;
    return;
  }
  // columns before c are not read again, so the swap and the division cover
  // columns c..n
  for (int j = c + threadIdx.x; j <= n; j += 256) {
    const double x = a[(long long)c * w + j], y = a[(long long)im * w + j];
    a[(long long)im * w + j] = x;
    a[(long long)c * w + j] = y / f;
  }
}

// Every row r != c of pair d: a[r][j] -= a[r][c] a[c][j] for j in (c, n];
// column c itself is not read again and is left as it is.
__global__ void __launch_bounds__(256)
    lm_eliminate(int n, int c, double* __restrict__ aug, const int* __restrict__ singular) {
  const int d = blockIdx.z;
  if (singular[d]) return;
  const long long w = n + 1;
  double* a = aug + (long long)d * n * w;
  const int r = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (r >= n || r == c) return;
  const double m = a[(long long)r * w + c];
  if (m == 0.0) return;
  for (int j = c + 1 + blockIdx.x * 32 + (threadIdx.x & 31); j <= n; j += gridDim.x * 32)
    a[(long long)r * w + j] = fma(-m, a[(long long)c * w + j], a[(long long)r * w + j]);
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
    // up to eight 32-column blocks per 8-row block (one warp per row, looping
    // over the row's remaining columns, measured 13% slower at n = 2700)
    const unsigned gx = (unsigned)std::max<size_t>(1, std::min<size_t>(8, (n + 1 + 31) / 32));
    for (int col = 0; col < ncols; col++) {
      lm_pivot<<<nd, 256, 0, c->stream>>>(ncols, col, aug, singular);
      lm_eliminate<<<dim3(gx, (unsigned)((n + 7) / 8), nd), 256, 0, c->stream>>>(ncols, col, aug,
                                                                                 singular);
    }
    lm_finish<<<(unsigned)(((size_t)nd * n + 255) / 256), 256, 0, c->stream>>>(
        ncols, nd, aug, singular, (const double*)pb, oB);
  }
  c->launches += 4 + 2LL * ncols;
  if ((rc = ztm_after_launch(c, "normal equations"))) return rc;
  if (!dev) {
    if (JJ) cudaMemcpyAsync(JJ, oJJ, n * n * 8, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(B, oB, (size_t)nd * n * 8, cudaMemcpyDeviceToHost, c->stream);
  }
  return ztm_finish(c, dev, nullptr, nullptr, 0, "normal equations");
}
