/*
 * oracle.c - CPU oracle of the gravity path.  TEST INFRASTRUCTURE ONLY: the
 * tests, the smoke check and the bench's CPU-baseline leg load it to check
 * results against; the product library never links it and has no CPU
 * fallback.
 *
 * Point-mass model (the reference's algorithm):
 *   ora_pointmass_tfm  restates the CPU gravity lambda of TFM.cpp:95-99 with
 *                      its index maps (TFM.cpp:85,97), its bfr interior
 *                      (TFM.cpp:96,99), pow(.,1.5) in double, summation in
 *                      nn order and the per-term division by fh*fh*fv.  The
 *                      reference gives each station row a thread; here the
 *                      threads split the stations evenly (same arithmetic per
 *                      station), so that a bounded sample of stations still
 *                      uses every core.
 *   ora_pointmass_adjoint  the transpose of that sum (no counterpart in the
 *                      reference, whose optimiser differentiates by finite
 *                      differences, TFM.cpp:124-135): per node, the weighted
 *                      sum over stations of the same per-pair term.
 *   ora_pointmass_gf   restates the GF kernel of GFM_GPU.cu:16-22 in float,
 *                      with the kernel's own index math (ii=di*fh, :17) and a
 *                      sequential (thread-order) summation in place of the
 *                      unordered atomicAdd.
 * Prism model (no reference code exists; published closed form):
 *   gz = G*rho * sum_{corners} s_x s_y s_z * Phi(x, y, z),
 *   Phi = x ln(y+r) + y ln(x+r) - z atan(x y / (z r)),
 * with corner coordinates taken mass-minus-station, z up, and s = +1 at the
 * upper and -1 at the lower limit of each axis (Nagy 1966; Plouff 1976;
 * Nagy, Papp & Benedek 2000, J. Geodesy 74:552).  The top-face derivative
 * used by the interface adjoint is the 4-corner sum of atan(x y / (w r)),
 * w = z_station - z_face.
 *
 * Parity is pinned for the point-mass model by the GF kernel's own outputs
 * (tests/golden) and for the prism model by mathematical known answers in the
 * tests (quadrature, Bouguer slab, superposition, far-field point-mass limit).
 *
 * Built with -ffp-contract=off so that x86 and aarch64 hosts round alike.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MGAL 1.0e5

/* ---------------------------------------------------------------------- */
/* minimal parallel-for                                                    */
typedef void (*range_fn)(long lo, long hi, void* arg);
typedef struct {
  range_fn fn;
  void* arg;
  long lo, hi;
} task_t;

static void* task_run(void* p) {
  task_t* t = (task_t*)p;
  t->fn(t->lo, t->hi, t->arg);
  return NULL;
}

static void parallel_for(long n, int nthreads, range_fn fn, void* arg) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (n < nthreads) nthreads = (int)(n > 0 ? n : 1);
  if (nthreads == 1) {
    fn(0, n, arg);
    return;
  }
  pthread_t th[256];
  task_t tk[256];
  long per = (n + nthreads - 1) / nthreads;
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    long lo = t * per, hi = lo + per < n ? lo + per : n;
    if (lo >= hi) break;
    tk[t].fn = fn;
    tk[t].arg = arg;
    tk[t].lo = lo;
    tk[t].hi = hi;
    if (pthread_create(&th[t], NULL, task_run, &tk[t]) != 0) {
      fn(lo, hi, arg); /* could not spawn: run inline */
      tk[t].fn = NULL;
    }
    started++;
  }
  for (int t = 0; t < started; t++)
    if (tk[t].fn) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------------- */
/* point-mass model                                                        */
typedef struct {
  int di, dj, dk, fh, fv, bfr, ii, jj, ni;
  long s_lo;
  const double* drho;
  const int* nn;
  long n_nn;
  const double* surf;
  double* G;
} pm_args;

/* Interior stations s_lo+lo .. s_lo+hi (row-major over (i0, j0)); each
 * station is the body of the GFM lambda of TFM.cpp:96-98 for one i0. */
static void pm_stations(long lo, long hi, void* p) {
  pm_args* a = (pm_args*)p;
  const int fh = a->fh, fv = a->fv, ii = a->ii, jj = a->jj;
  for (long t = lo; t < hi; t++) {
    long sidx = a->s_lo + t;
    int i0 = a->bfr + (int)(sidx % a->ni), j0 = a->bfr + (int)(sidx / a->ni);
    int m = i0 + j0 * a->di;
    double k0 = a->surf[m];
    double g = 0;
    for (long q = 0; q < a->n_nn; q++) {
      int n = a->nn[q];
      double i = (n % ii) / (1. * fh), j = ((n / ii) % jj) / (1. * fh),
             k = (n / (ii * jj)) / (1. * fv);
      g += (66.7 * a->drho[n] * (k0 - k) /
            pow((i0 - i) * (i0 - i) + (j0 - j) * (j0 - j) + (k0 - k) * (k0 - k), 1.5)) /
           (fh * fh * fv);
    }
    a->G[m] = g;
  }
}

void ora_pointmass_tfm_range(int di, int dj, int dk, int fh, int fv, int bfr,
                             const double* drho, const int* nn, long n_nn,
                             const double* surf, double* G, long s_lo, long s_hi,
                             int nthreads) {
  pm_args a;
  a.di = di; a.dj = dj; a.dk = dk; a.fh = fh; a.fv = fv; a.bfr = bfr;
  a.ii = (di - 1) * fh + 1;
  a.jj = (dj - 1) * fh + 1;
  a.ni = di - 2 * bfr;
  a.drho = drho; a.nn = nn; a.n_nn = n_nn; a.surf = surf; a.G = G;
  long ns = (long)(di - 2 * bfr) * (dj - 2 * bfr);
  if (di - 2 * bfr <= 0 || dj - 2 * bfr <= 0) return;
  if (s_hi < 0 || s_hi > ns) s_hi = ns;
  if (s_lo < 0) s_lo = 0;
  if (s_hi <= s_lo) return;
  a.s_lo = s_lo;
  parallel_for(s_hi - s_lo, nthreads, pm_stations, &a);
}

void ora_pointmass_tfm(int di, int dj, int dk, int fh, int fv, int bfr,
                       const double* drho, const int* nn, long n_nn,
                       const double* surf, double* G, int nthreads) {
  ora_pointmass_tfm_range(di, dj, dk, fh, fv, bfr, drho, nn, n_nn, surf, G, 0, -1, nthreads);
}

/* Transpose of the TFM.cpp:96-98 sum: for every entry q of the node list,
 * gq = sum over interior stations (j0 outer, i0 inner, as the lambda's rows
 * and columns) of w[m] * 66.7*(k0-k)/pow(r^2,1.5)/(fh*fh*fv); the entries are
 * then added into g[nn[q]] in list order (a node listed twice gets it twice),
 * so that sum_m w[m] G[m] = sum_n g[n] drho[n] for the forward over the same
 * list. */
typedef struct {
  int di, dj, fh, fv, bfr, ii, jj;
  const int* nn;
  const double* surf;
  const double* w;
  double* gq;
} pma_args;

static void pma_entries(long lo, long hi, void* p) {
  pma_args* a = (pma_args*)p;
  const int fh = a->fh, fv = a->fv, ii = a->ii, jj = a->jj;
  for (long q = lo; q < hi; q++) {
    int n = a->nn[q];
    double i = (n % ii) / (1. * fh), j = ((n / ii) % jj) / (1. * fh), k = (n / (ii * jj)) / (1. * fv);
    double g = 0;
    for (int j0 = a->bfr; j0 < a->dj - a->bfr; j0++)
      for (int i0 = a->bfr; i0 < a->di - a->bfr; i0++) {
        int m = i0 + j0 * a->di;
        double k0 = a->surf[m];
        g += a->w[m] * (66.7 * (k0 - k) /
                        pow((i0 - i) * (i0 - i) + (j0 - j) * (j0 - j) + (k0 - k) * (k0 - k), 1.5)) /
             (fh * fh * fv);
      }
    a->gq[q] = g;
  }
}

void ora_pointmass_adjoint(int di, int dj, int dk, int fh, int fv, int bfr, const int* nn,
                           long n_nn, const double* surf, const double* w, double* g, int nthreads) {
  long N = (long)((di - 1) * fh + 1) * ((dj - 1) * fh + 1) * ((dk - 1) * fv + 1);
  memset(g, 0, sizeof(double) * N);
  if (di - 2 * bfr <= 0 || dj - 2 * bfr <= 0 || n_nn <= 0) return;
  pma_args a;
  a.di = di; a.dj = dj; a.fh = fh; a.fv = fv; a.bfr = bfr;
  a.ii = (di - 1) * fh + 1;
  a.jj = (dj - 1) * fh + 1;
  a.nn = nn; a.surf = surf; a.w = w;
  a.gq = (double*)malloc(sizeof(double) * n_nn);
  if (!a.gq) return;
  parallel_for(n_nn, nthreads, pma_entries, &a);
  for (long q = 0; q < n_nn; q++) g[nn[q]] += a.gq[q];
  free(a.gq);
}

void ora_pointmass_gf(int bfr, int di, int dj, int dk, int fh, int fv,
                      const float* rho, long nthreads_total, const float* s,
                      float* g) {
  (void)dk; /* the kernel never reads dk (GFM_GPU.cu:17-18) */
  float c = 66.7f / (fh * fh * fv);
  int ii = di * fh, jj = dj * fh;
  for (long n = 0; n < nthreads_total; n++) {
    float i = (n % ii) * 1.f / fh, j = ((n / ii) % jj) * 1.f / fh,
          k = (n / (ii * jj)) * 1.f / fv;
    if (fabsf(rho[n]) > .001f) {
      for (int ni = bfr; ni < di - bfr; ni++) {
        for (int nj = bfr; nj < dj - bfr; nj++) {
          int m = ni + nj * di;
          float i0 = ni, j0 = nj, k0 = s[m];
          g[m] += c * rho[n] * (k0 - k) /
                  powf((i0 - i) * (i0 - i) + (j0 - j) * (j0 - j) +
                           (k0 - k) * (k0 - k),
                       1.5f);
        }
      }
    }
  }
}

/* ---------------------------------------------------------------------- */
/* prism model                                                             */

/* x*ln(y+r) with the y<0 branch rewritten as x*ln((x^2+z^2)/(r-y)) so that
 * y+r never cancels; 0 when x == 0 (the 0*ln 0 limit). */
static double xlog(double x, double y, double z, double r) {
  if (x == 0.0) return 0.0;
  if (y >= 0.0) return x * log(y + r);
  return x * log((x * x + z * z) / (r - y));
}

double ora_phi(double x, double y, double z) {
  double r = sqrt(x * x + y * y + z * z);
  if (r == 0.0) return 0.0;
  double t = xlog(x, y, z, r) + xlog(y, x, z, r);
  if (z != 0.0) t -= z * atan(x * y / (z * r));
  return t;
}

static long double xlogl(long double x, long double y, long double z,
                         long double r) {
  if (x == 0.0L) return 0.0L;
  if (y >= 0.0L) return x * logl(y + r);
  return x * logl((x * x + z * z) / (r - y));
}

long double ora_phil(long double x, long double y, long double z) {
  long double r = sqrtl(x * x + y * y + z * z);
  if (r == 0.0L) return 0.0L;
  long double t = xlogl(x, y, z, r) + xlogl(y, x, z, r);
  if (z != 0.0L) t -= z * atanl(x * y / (z * r));
  return t;
}

/* Integral of (zs - z)/r^3 over the prism, i.e. gz / (G*rho). */
double ora_prism_unit(double xs, double ys, double zs, double x0, double x1,
                      double y0, double y1, double z0, double z1) {
  double xa[2] = {x0 - xs, x1 - xs}, ya[2] = {y0 - ys, y1 - ys},
         za[2] = {z0 - zs, z1 - zs};
  double s = 0.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 2; c++) {
        /* s_x s_y s_z = (-1)^(number of lower limits) */
        double sg = ((a + b + c) & 1) ? 1.0 : -1.0;
        s += sg * ora_phi(xa[a], ya[b], za[c]);
      }
  return s;
}

long double ora_prism_unitl(long double xs, long double ys, long double zs,
                            long double x0, long double x1, long double y0,
                            long double y1, long double z0, long double z1) {
  long double xa[2] = {x0 - xs, x1 - xs}, ya[2] = {y0 - ys, y1 - ys},
              za[2] = {z0 - zs, z1 - zs};
  long double s = 0.0L;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++)
      for (int c = 0; c < 2; c++) {
        long double sg = ((a + b + c) & 1) ? 1.0L : -1.0L;
        s += sg * ora_phil(xa[a], ya[b], za[c]);
      }
  return s;
}

/* Integral of w/r^3 over the horizontal face z = zf, w = zs - zf. */
double ora_face_unit(double xs, double ys, double zs, double x0, double x1,
                     double y0, double y1, double zf) {
  double w = zs - zf;
  if (w == 0.0) return 0.0;
  double xa[2] = {x0 - xs, x1 - xs}, ya[2] = {y0 - ys, y1 - ys};
  double s = 0.0;
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      double sg = (a == b) ? 1.0 : -1.0;
      double x = xa[a], y = ya[b];
      double r = sqrt(x * x + y * y + w * w);
      s += sg * atan(x * y / (w * r));
    }
  return s;
}

typedef struct {
  const double* mp;
  const double* rho;
  const double* sxyz;
  double G;
  double* out;
  int use_ld;
  const double* resid;
  int ns;
  long np;
  const double* geom;
  const double* depth;
  double* out2;
} pr_args;

static void prism_mesh_rows(long lo, long hi, void* p) {
  pr_args* a = (pr_args*)p;
  const double* m = a->mp;
  int nx = (int)m[0], ny = (int)m[1], nz = (int)m[2];
  double x0 = m[3], y0 = m[4], zt = m[5], dx = m[6], dy = m[7], dz = m[8];
  for (long s = lo; s < hi; s++) {
    double xs = a->sxyz[3 * s], ys = a->sxyz[3 * s + 1], zs = a->sxyz[3 * s + 2];
    double acc = 0.0;
    long double accl = 0.0L;
    for (int l = 0; l < nz; l++) {
      double za = zt - (l + 1) * dz, zb = zt - l * dz;
      for (int iy = 0; iy < ny; iy++) {
        double ya = y0 + iy * dy, yb = y0 + (iy + 1) * dy;
        for (int ix = 0; ix < nx; ix++) {
          double r = a->rho[ix + (long)nx * (iy + (long)ny * l)];
          if (r == 0.0) continue;
          double xa = x0 + ix * dx, xb = x0 + (ix + 1) * dx;
          if (a->use_ld)
            accl += (long double)r * ora_prism_unitl(xs, ys, zs, xa, xb, ya, yb, za, zb);
          else
            acc += r * ora_prism_unit(xs, ys, zs, xa, xb, ya, yb, za, zb);
        }
      }
    }
    a->out[s] = a->use_ld ? (double)(accl * a->G * MGAL) : acc * a->G * MGAL;
  }
}

void ora_prism_mesh(const double* mp, const double* rho, int ns,
                    const double* sxyz, double G, double* gz, int nthreads,
                    int use_long_double) {
  pr_args a;
  memset(&a, 0, sizeof a);
  a.mp = mp; a.rho = rho; a.sxyz = sxyz; a.G = G; a.out = gz;
  a.use_ld = use_long_double;
  parallel_for(ns, nthreads, prism_mesh_rows, &a);
}

static void prism_list_rows(long lo, long hi, void* p) {
  pr_args* a = (pr_args*)p;
  for (long s = lo; s < hi; s++) {
    double xs = a->sxyz[3 * s], ys = a->sxyz[3 * s + 1], zs = a->sxyz[3 * s + 2];
    double acc = 0.0;
    for (long q = 0; q < a->np; q++) {
      const double* g = a->geom + 6 * q;
      if (a->rho[q] == 0.0) continue;
      acc += a->rho[q] * ora_prism_unit(xs, ys, zs, g[0], g[1], g[2], g[3], g[4], g[5]);
    }
    a->out[s] = acc * a->G * MGAL;
  }
}

void ora_prism_list(long np, const double* geom, const double* rho, int ns,
                    const double* sxyz, double G, double* gz, int nthreads) {
  pr_args a;
  memset(&a, 0, sizeof a);
  a.np = np; a.geom = geom; a.rho = rho; a.sxyz = sxyz; a.G = G; a.out = gz;
  parallel_for(ns, nthreads, prism_list_rows, &a);
}

/* g_rho[p] = sum_s resid[s] * G * unit(s, p), one prism per iteration. */
static void mesh_adj_rows(long lo, long hi, void* p) {
  pr_args* a = (pr_args*)p;
  const double* m = a->mp;
  int nx = (int)m[0], ny = (int)m[1];
  double x0 = m[3], y0 = m[4], zt = m[5], dx = m[6], dy = m[7], dz = m[8];
  for (long q = lo; q < hi; q++) {
    int ix = (int)(q % nx), iy = (int)((q / nx) % ny), l = (int)(q / ((long)nx * ny));
    double xa = x0 + ix * dx, xb = x0 + (ix + 1) * dx;
    double ya = y0 + iy * dy, yb = y0 + (iy + 1) * dy;
    double za = zt - (l + 1) * dz, zb = zt - l * dz;
    double acc = 0.0;
    for (int s = 0; s < a->ns; s++) {
      double u = ora_prism_unit(a->sxyz[3 * s], a->sxyz[3 * s + 1], a->sxyz[3 * s + 2],
                                xa, xb, ya, yb, za, zb);
      acc += a->resid[s] * u;
    }
    a->out[q] = acc * a->G * MGAL;
  }
}

void ora_mesh_adjoint(const double* mp, int ns, const double* sxyz,
                      const double* resid, double G, double* g_rho,
                      int nthreads) {
  pr_args a;
  memset(&a, 0, sizeof a);
  a.mp = mp; a.sxyz = sxyz; a.resid = resid; a.G = G; a.out = g_rho; a.ns = ns;
  long np = (long)mp[0] * (long)mp[1] * (long)mp[2];
  parallel_for(np, nthreads, mesh_adj_rows, &a);
}

/* ---------------------------------------------------------------------- */
/* interface (column) model                                                */
static void iface_fwd_rows(long lo, long hi, void* p) {
  pr_args* a = (pr_args*)p;
  const double* m = a->mp;
  int nx = (int)m[0], ny = (int)m[1];
  double x0 = m[2], y0 = m[3], dx = m[4], dy = m[5], zb = m[6];
  for (long s = lo; s < hi; s++) {
    double xs = a->sxyz[3 * s], ys = a->sxyz[3 * s + 1], zs = a->sxyz[3 * s + 2];
    double acc = 0.0;
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        long c = ix + (long)nx * iy;
        double r = a->rho[c];
        if (r == 0.0) continue;
        acc += r * ora_prism_unit(xs, ys, zs, x0 + ix * dx, x0 + (ix + 1) * dx,
                                  y0 + iy * dy, y0 + (iy + 1) * dy, zb, -a->depth[c]);
      }
    a->out[s] = acc * a->G * MGAL;
  }
}

void ora_interface_fwd(const double* imp, const double* depth,
                       const double* rho_col, int ns, const double* sxyz,
                       double G, double* gz, int nthreads) {
  pr_args a;
  memset(&a, 0, sizeof a);
  a.mp = imp; a.depth = depth; a.rho = rho_col; a.sxyz = sxyz; a.G = G; a.out = gz;
  parallel_for(ns, nthreads, iface_fwd_rows, &a);
}

/* d gz / d depth = -G rho * face(top); d gz / d rho = G * unit. */
static void iface_adj_rows(long lo, long hi, void* p) {
  pr_args* a = (pr_args*)p;
  const double* m = a->mp;
  int nx = (int)m[0];
  double x0 = m[2], y0 = m[3], dx = m[4], dy = m[5], zb = m[6];
  for (long c = lo; c < hi; c++) {
    int ix = (int)(c % nx), iy = (int)(c / nx);
    double xa = x0 + ix * dx, xb = x0 + (ix + 1) * dx;
    double ya = y0 + iy * dy, yb = y0 + (iy + 1) * dy;
    double zt = -a->depth[c];
    double gr = 0.0, gd = 0.0;
    for (int s = 0; s < a->ns; s++) {
      double xs = a->sxyz[3 * s], ys = a->sxyz[3 * s + 1], zs = a->sxyz[3 * s + 2];
      double res = a->resid[s];
      if (a->out) gr += res * ora_prism_unit(xs, ys, zs, xa, xb, ya, yb, zb, zt);
      if (a->out2) gd += res * ora_face_unit(xs, ys, zs, xa, xb, ya, yb, zt);
    }
    if (a->out) a->out[c] = gr * a->G * MGAL;
    if (a->out2) a->out2[c] = -gd * a->rho[c] * a->G * MGAL;
  }
}

void ora_interface_adj(const double* imp, const double* depth,
                       const double* rho_col, int ns, const double* sxyz,
                       const double* resid, double G, double* g_rho,
                       double* g_depth, int nthreads) {
  pr_args a;
  memset(&a, 0, sizeof a);
  a.mp = imp; a.depth = depth; a.rho = rho_col; a.sxyz = sxyz; a.resid = resid;
  a.G = G; a.out = g_rho; a.out2 = g_depth; a.ns = ns;
  long nc = (long)imp[0] * (long)imp[1];
  parallel_for(nc, nthreads, iface_adj_rows, &a);
}

/* ---------------------------------------------------------------------- */
/* density-perturbation builder (TFM.cpp:83-89)                            */

/* zmath.cpp:225-235, 2-D linear interpolation with unit spacing.  The
 * reference reads f[i+1] / f[(j+1)*di] even when the weight of that
 * neighbour is 0 (x = di-1 or y = dj-1), one element past the row or the
 * array; the index is clamped here, which changes nothing but the read. */
static double interp2_tfm(const double* f, double x, double y, int di, int dj) {
  double ii = fmin(fmax(x / 1.0, 0), (di - 1)), jj = fmin(fmax(y / 1.0, 0), (dj - 1));
  int i = (int)ii, j = (int)jj;
  double si = ii - i, sj = jj - j;
  int i1 = i + 1 < di ? i + 1 : i, j1 = j + 1 < dj ? j + 1 : j;
  double c00 = f[i + j * di], c10 = f[i1 + j * di];
  double c01 = f[i + j1 * di], c11 = f[i1 + j1 * di];
  double c0 = c00 * (1 - si) + c10 * si, c1 = c01 * (1 - si) + c11 * si;
  return c0 * (1 - sj) + c1 * sj;
}

/* zmath.cpp:238-252, 3-D linear interpolation with unit spacing. */
static double interp3_tfm(const double* f, double x, double y, double z, int di, int dj,
                          int dk) {
  double ii = fmin(fmax(x / 1.0, 0), (di - 2)), jj = fmin(fmax(y / 1.0, 0), (dj - 2)),
         kk = fmin(fmax(z / 1.0, 0), (dk - 2));
  int i = (int)ii, j = (int)jj, k = (int)kk;
  double si = ii - i, sj = jj - j, sk = kk - k;
  long p = (long)di * dj;
  double c000 = f[i + j * di + k * p], c100 = f[i + 1 + j * di + k * p];
  double c010 = f[i + (j + 1) * di + k * p], c110 = f[i + 1 + (j + 1) * di + k * p];
  double c001 = f[i + j * di + (k + 1) * p], c101 = f[i + 1 + j * di + (k + 1) * p];
  double c011 = f[i + (j + 1) * di + (k + 1) * p], c111 = f[i + 1 + (j + 1) * di + (k + 1) * p];
  double c00 = c000 * (1 - si) + c100 * si, c01 = c001 * (1 - si) + c101 * si;
  double c10 = c010 * (1 - si) + c110 * si, c11 = c011 * (1 - si) + c111 * si;
  double c0 = c00 * (1 - sj) + c10 * sj, c1 = c01 * (1 - sj) + c11 * sj;
  return c0 * (1 - sk) + c1 * sk;
}

/* Depth (km) of grid point (i, j, k): c2g of TFM.cpp:56 through enu2geo of
 * SET.cpp:86-99 (ECEF rotation about the reference, r by sqrtf).  g holds
 * the reference-point terms: m[9], xr, yr, zr, then RC[3], RC[4], RC[5],
 * RC[6]. */
static double depth_tfm(const double* g, double i, double j, double k) {
  const double* m = g;
  double x = i * g[15] - g[12], y = j * g[15] - g[13], z = k * g[15] - g[14];
  double xi = m[0] * x + m[1] * y + m[2] * z + g[9];
  double yi = m[3] * x + m[4] * y + m[5] * z + g[10];
  double zi = m[6] * x + m[7] * y + m[8] * z + g[11];
  double r = sqrtf(xi * xi + yi * yi + zi * zi);
  return 6371 - r;
}

/* The reference-point terms of enu2geo (SET.cpp:87-93) for RC. */
void ora_density_geo(const double* rc, double* g) {
  double rad = 57.295, R = 6371;
  double lat_ref = rc[0], lon_ref = rc[1], d_ref = rc[2];
  double phi = lat_ref / rad, theta = lon_ref / rad;
  double m[9] = {-sin(theta), -sin(phi) * cos(theta), cos(phi) * cos(theta),
                 cos(theta),  -sin(phi) * sin(theta), cos(phi) * sin(theta),
                 0,           cos(phi),               sin(phi)};
  for (int t = 0; t < 9; t++) g[t] = m[t];
  g[9] = (R - d_ref) * cos(lon_ref / rad) * cos(lat_ref / rad);
  g[10] = (R - d_ref) * sin(lon_ref / rad) * cos(lat_ref / rad);
  g[11] = (R - d_ref) * sin(lat_ref / rad);
  g[12] = rc[3];
  g[13] = rc[4];
  g[14] = rc[5];
  g[15] = rc[6];
}

typedef struct {
  int di, dj, dk, fh, fv, ii, jj;
  double vm, ro, dr;
  const double *sea, *M, *v, *geo;
  double* drho;
} dens_args;

static void dens_rows(long lo, long hi, void* p) {
  dens_args* a = (dens_args*)p;
  const int fh = a->fh, fv = a->fv, ii = a->ii, jj = a->jj;
  for (long n = lo; n < hi; n++) {
    double i = (n % ii) / (1. * fh), j = ((n / ii) % jj) / (1. * fh),
           k = (n / ((long)ii * jj)) / (1. * fv), li = 1. / fv, m0, m1, r0, r1;
    m0 = interp2_tfm(a->sea, i, j, a->di, a->dj) - 3.5;
    m1 = interp2_tfm(a->M, i, j, a->di, a->dj);
    r0 = 0;
    r1 = a->dr * (interp3_tfm(a->v, i, j, k, a->di, a->dj, a->dk) - a->vm);
    if (k > m0 + li) {
      r0 = a->ro;
    } else if (fabs(k - m0) < li) {
      r0 = r0 + (k - m0 + li) * (r0 + a->ro) / (2 * li);
    }
    if (k > m1 + li) {
      r1 = a->ro;
    } else if (fabs(k - m1) < li) {
      r1 = r1 + (k - m1 + li) * (r1 + a->ro) / (2 * li);
    }
    a->drho[n] = (fabs(r0 - r1) > .001 && depth_tfm(a->geo, i, j, k) > 10) ? r1 - r0 : 0.0;
  }
}

/* TFM.cpp:85-89: drho on the fine grid (zero where the node is not in nn). */
void ora_density_tfm(int di, int dj, int dk, int fh, int fv, double vm, double ro, double dr,
                     const double* rc, const double* sea, const double* M, const double* v,
                     double* drho, int nthreads) {
  double geo[16];
  ora_density_geo(rc, geo);
  dens_args a;
  a.di = di; a.dj = dj; a.dk = dk; a.fh = fh; a.fv = fv;
  a.ii = (di - 1) * fh + 1;
  a.jj = (dj - 1) * fh + 1;
  a.vm = vm; a.ro = ro; a.dr = dr;
  a.sea = sea; a.M = M; a.v = v; a.geo = geo; a.drho = drho;
  long N = (long)a.ii * a.jj * ((dk - 1) * fv + 1);
  parallel_for(N, nthreads, dens_rows, &a);
}
