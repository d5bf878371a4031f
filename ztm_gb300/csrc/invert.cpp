// invert.cpp - nonlinear interface (Moho depth) inversion driven through the
// C ABI: every iteration runs the forward and the adjoint on the GPU
// (ztm_gfm_interface_misfit) and the optimiser on the host.
//
// Objective, with m = depth in km (column tops) and r = gz(m) - data:
//   phi(m) = 0.5 |r|^2 + 0.5 * lambda * sum over neighbouring columns of
//            (m_i - m_j)^2            (first-order Tikhonov smoothing)
// minimised by L-BFGS (two-loop recursion, history 8) with a backtracking
// Armijo line search (ztm_invert_interface), or by Gauss-Newton with
// conjugate-gradient inner solves whose Hessian products are one J v
// (ztm_gfm_interface_jvp) and one J^T w (the depth adjoint) each
// (ztm_invert_interface_gn); depths kept inside [0, -z_base] by projection.
//
// The reference's optimiser is a damped Gauss-Newton (Levenberg-Marquardt)
// over a grid of damping factors (TFM.cpp:155-167) whose gravity Jacobian
// columns come from one full forward per parameter (TFM.cpp:124-135); the
// adjoint gradient replaces those columns, so an iteration costs one
// forward and one adjoint whatever the number of depth parameters.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ztm_grav.h"

namespace {

struct Problem {
  ztm_ctx* ctx;
  const ztm_imesh* mesh;
  const double* rho;
  int ns;
  const double* sxyz;
  const double* data;
  double lambda;
  ztm_opts opts;
  int nx, ny;
  long long evals = 0;
};

// phi and its gradient (per km) at depth m (km).
int evaluate(Problem& P, const std::vector<double>& m, double* f, std::vector<double>& g,
             double* data_misfit) {
  const size_t nc = m.size();
  std::vector<double> dm(nc), g_dep(nc);
  for (size_t c = 0; c < nc; c++) dm[c] = 1000.0 * m[c];
  double mis = 0.0;
  int rc = ztm_gfm_interface_misfit(P.ctx, P.mesh, dm.data(), P.rho, P.ns, P.sxyz, P.data, &mis,
                                    nullptr, nullptr, g_dep.data(), &P.opts);
  if (rc) return rc;
  P.evals++;
  double reg = 0.0;
  g.assign(nc, 0.0);
  for (size_t c = 0; c < nc; c++) g[c] = 1000.0 * g_dep[c];  // d/dm (km) = 1000 d/ddepth (m)
  for (int iy = 0; iy < P.ny; iy++)
    for (int ix = 0; ix < P.nx; ix++) {
      const size_t c = ix + (size_t)P.nx * iy;
      if (ix + 1 < P.nx) {
        const double d = m[c] - m[c + 1];
        reg += d * d;
        g[c] += P.lambda * d;
        g[c + 1] -= P.lambda * d;
      }
      if (iy + 1 < P.ny) {
        const double d = m[c] - m[c + P.nx];
        reg += d * d;
        g[c] += P.lambda * d;
        g[c + P.nx] -= P.lambda * d;
      }
    }
  *f = mis + 0.5 * P.lambda * reg;
  if (data_misfit) *data_misfit = mis;
  return ZTM_OK;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}

// out += lambda * L v: the Hessian of the smoothing term (graph Laplacian of
// the column grid, first-order differences).
void add_smoothing_hessian(const Problem& P, const std::vector<double>& v, std::vector<double>& out) {
  for (int iy = 0; iy < P.ny; iy++)
    for (int ix = 0; ix < P.nx; ix++) {
      const size_t c = ix + (size_t)P.nx * iy;
      if (ix + 1 < P.nx) {
        const double d = P.lambda * (v[c] - v[c + 1]);
        out[c] += d;
        out[c + 1] -= d;
      }
      if (iy + 1 < P.ny) {
        const double d = P.lambda * (v[c] - v[c + P.nx]);
        out[c] += d;
        out[c + P.nx] -= d;
      }
    }
}

// Gauss-Newton Hessian product at depth m (km): (J^T J + lambda L) v, with J
// the depth derivative of the forward per km (ztm_gfm_interface_jvp for J v,
// the depth adjoint for J^T w; one of each per product).
int gn_product(Problem& P, const std::vector<double>& m, const std::vector<double>& v,
               std::vector<double>& out) {
  const size_t nc = m.size();
  std::vector<double> dm(nc), dv(nc), g_dep(nc), jv(P.ns);
  for (size_t c = 0; c < nc; c++) {
    dm[c] = 1000.0 * m[c];
    dv[c] = 1000.0 * v[c];  // km -> m
  }
  int rc = ztm_gfm_interface_jvp(P.ctx, P.mesh, dm.data(), P.rho, dv.data(), P.ns, P.sxyz,
                                 jv.data(), &P.opts);
  if (rc) return rc;
  rc = ztm_gfm_interface_adjoint(P.ctx, P.mesh, dm.data(), P.rho, P.ns, P.sxyz, jv.data(), nullptr,
                                 g_dep.data(), &P.opts);
  if (rc) return rc;
  P.evals++;
  out.assign(nc, 0.0);
  for (size_t c = 0; c < nc; c++) out[c] = 1000.0 * g_dep[c];
  add_smoothing_hessian(P, v, out);
  return ZTM_OK;
}

}  // namespace

extern "C" int ztm_invert_interface(ztm_ctx* ctx, const ztm_imesh* mesh, double* depth,
                                    const double* rho_col, int ns, const double* sxyz,
                                    const double* data, double lambda, int iterations,
                                    const ztm_opts* opt, double* history, int* n_done) {
  if (!ctx || !mesh || !depth || !rho_col || !sxyz || !data || ns < 1 || iterations < 0 ||
      !(lambda >= 0))
    return ZTM_ERR_ARG;
  if (opt && (opt->flags & ZTM_FLAG_DEVICE_PTRS)) return ZTM_ERR_ARG;  // host arrays only
  Problem P;
  P.ctx = ctx;
  P.mesh = mesh;
  P.rho = rho_col;
  P.ns = ns;
  P.sxyz = sxyz;
  P.data = data;
  P.lambda = lambda;
  memset(&P.opts, 0, sizeof P.opts);
  if (opt) P.opts = *opt;
  P.nx = mesh->nx;
  P.ny = mesh->ny;
  const size_t nc = (size_t)mesh->nx * mesh->ny;
  const double dmax = -mesh->z_base / 1000.0;  // tops stay above the bases
  std::vector<double> m(nc), g(nc), mt(nc), gt(nc), d(nc);
  for (size_t c = 0; c < nc; c++) m[c] = std::min(std::max(depth[c] / 1000.0, 0.0), dmax);
  double f = 0.0, mis = 0.0;
  int rc = evaluate(P, m, &f, g, &mis);
  if (rc) return rc;
  const int H = 8;
  std::vector<std::vector<double>> S, Y;
  std::vector<double> rhoh;
  int it = 0;
  for (; it < iterations; it++) {
    if (history) history[it] = mis;
    // two-loop recursion: d = -H g
    d = g;
    std::vector<double> alpha(S.size());
    for (int k = (int)S.size() - 1; k >= 0; k--) {
      alpha[k] = rhoh[k] * dot(S[k], d);
      for (size_t i = 0; i < nc; i++) d[i] -= alpha[k] * Y[k][i];
    }
    double gamma;
    if (!S.empty()) {
      gamma = dot(S.back(), Y.back()) / dot(Y.back(), Y.back());
    } else {
      double gn = sqrt(dot(g, g));
      gamma = gn > 0 ? 1.0 / gn : 1.0;  // first step: 1 km along -g/|g|
    }
    for (size_t i = 0; i < nc; i++) d[i] *= gamma;
    for (int k = 0; k < (int)S.size(); k++) {
      const double beta = rhoh[k] * dot(Y[k], d);
      for (size_t i = 0; i < nc; i++) d[i] += S[k][i] * (alpha[k] - beta);
    }
    for (size_t i = 0; i < nc; i++) d[i] = -d[i];
    double slope = dot(g, d);
    if (!(slope < 0)) {  // not a descent direction: restart on steepest descent
      S.clear();
      Y.clear();
      rhoh.clear();
      double gn = sqrt(dot(g, g));
      if (gn == 0) break;
      for (size_t i = 0; i < nc; i++) d[i] = -g[i] / gn;
      slope = dot(g, d);
    }
    // backtracking Armijo line search with projection
    double step = 1.0, ft = 0.0, mist = 0.0;
    bool accepted = false;
    for (int ls = 0; ls < 20; ls++) {
      for (size_t i = 0; i < nc; i++) mt[i] = std::min(std::max(m[i] + step * d[i], 0.0), dmax);
      rc = evaluate(P, mt, &ft, gt, &mist);
      if (rc) return rc;
      if (ft <= f + 1e-4 * step * slope) {
        accepted = true;
        break;
      }
      step *= 0.5;
    }
    if (!accepted) break;
    std::vector<double> s(nc), y(nc);
    for (size_t i = 0; i < nc; i++) {
      s[i] = mt[i] - m[i];
      y[i] = gt[i] - g[i];
    }
    const double sy = dot(s, y);
    if (sy > 1e-12 * sqrt(dot(s, s) * dot(y, y))) {
      S.push_back(s);
      Y.push_back(y);
      rhoh.push_back(1.0 / sy);
      if ((int)S.size() > H) {
        S.erase(S.begin());
        Y.erase(Y.begin());
        rhoh.erase(rhoh.begin());
      }
    }
    m.swap(mt);
    g.swap(gt);
    f = ft;
    mis = mist;
  }
  if (history) history[it] = mis;
  if (n_done) *n_done = it;
  for (size_t c = 0; c < nc; c++) depth[c] = 1000.0 * m[c];
  return ZTM_OK;
}

// Gauss-Newton with conjugate-gradient inner solves: each iteration solves
// (J^T J + lambda L) d = -g for the step by at most cg_iterations CG steps
// (one J v and one J^T w on the GPU per step, J never formed), then takes
// the projected step with a backtracking line search on phi.  Same objective,
// units, bounds and history as ztm_invert_interface.
extern "C" int ztm_invert_interface_gn(ztm_ctx* ctx, const ztm_imesh* mesh, double* depth,
                                       const double* rho_col, int ns, const double* sxyz,
                                       const double* data, double lambda, int iterations,
                                       int cg_iterations, const ztm_opts* opt, double* history,
                                       int* n_done) {
  if (!ctx || !mesh || !depth || !rho_col || !sxyz || !data || ns < 1 || iterations < 0 ||
      cg_iterations < 1 || !(lambda >= 0))
    return ZTM_ERR_ARG;
  if (opt && (opt->flags & ZTM_FLAG_DEVICE_PTRS)) return ZTM_ERR_ARG;  // host arrays only
  Problem P;
  P.ctx = ctx;
  P.mesh = mesh;
  P.rho = rho_col;
  P.ns = ns;
  P.sxyz = sxyz;
  P.data = data;
  P.lambda = lambda;
  memset(&P.opts, 0, sizeof P.opts);
  if (opt) P.opts = *opt;
  P.nx = mesh->nx;
  P.ny = mesh->ny;
  const size_t nc = (size_t)mesh->nx * mesh->ny;
  const double dmax = -mesh->z_base / 1000.0;
  std::vector<double> m(nc), g(nc), mt(nc), gt(nc), x(nc), r(nc), p(nc), Ap(nc);
  for (size_t c = 0; c < nc; c++) m[c] = std::min(std::max(depth[c] / 1000.0, 0.0), dmax);
  double f = 0.0, mis = 0.0;
  int rc = evaluate(P, m, &f, g, &mis);
  if (rc) return rc;
  int it = 0;
  for (; it < iterations; it++) {
    if (history) history[it] = mis;
    // CG on (J^T J + lambda L) x = -g from x = 0
    std::fill(x.begin(), x.end(), 0.0);
    for (size_t i = 0; i < nc; i++) r[i] = -g[i];
    p = r;
    double rr = dot(r, r);
    const double rr0 = rr;
    if (rr0 == 0.0) break;
    for (int k = 0; k < cg_iterations; k++) {
      if ((rc = gn_product(P, m, p, Ap))) return rc;
      const double pAp = dot(p, Ap);
      if (!(pAp > 0)) break;
      const double alpha = rr / pAp;
      for (size_t i = 0; i < nc; i++) {
        x[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
      }
      const double rr1 = dot(r, r);
      if (rr1 <= 1e-12 * rr0) break;
      const double beta = rr1 / rr;
      rr = rr1;
      for (size_t i = 0; i < nc; i++) p[i] = r[i] + beta * p[i];
    }
    if (dot(x, g) >= 0) {  // not a descent step (CG broke down at once): steepest descent
      const double gn = sqrt(dot(g, g));
      for (size_t i = 0; i < nc; i++) x[i] = -g[i] / gn;
    }
    // projected step with backtracking
    double step = 1.0, ft = 0.0, mist = 0.0;
    bool accepted = false;
    for (int ls = 0; ls < 20; ls++) {
      for (size_t i = 0; i < nc; i++) mt[i] = std::min(std::max(m[i] + step * x[i], 0.0), dmax);
      if ((rc = evaluate(P, mt, &ft, gt, &mist))) return rc;
      if (ft < f) {
        accepted = true;
        break;
      }
      step *= 0.5;
    }
    if (!accepted) break;
    m.swap(mt);
    g.swap(gt);
    f = ft;
    mis = mist;
  }
  if (history) history[it] = mis;
  if (n_done) *n_done = it;
  for (size_t c = 0; c < nc; c++) depth[c] = 1000.0 * m[c];
  return ZTM_OK;
}
