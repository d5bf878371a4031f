/*
 * oracle.h - CPU restatement of ZTM's gravity path, used ONLY as the oracle
 * of the tests, the smoke check and the bench's CPU baseline.  Nothing in the
 * product library links or calls it.
 *
 * Parity pins: the point-mass functions restate TFM.cpp:95-99 (double) and
 * GFM_GPU.cu:16-22 (float) and are checked against outputs of the reference
 * GF kernel itself (tests/golden).  The prism, face and interface functions
 * have no reference implementation (ZTM has only the point-mass model); they
 * are pinned by mathematical known answers (numerical quadrature, Bouguer
 * slab, superposition, far-field limit to the point-mass model).
 */
#ifndef ZTM_ORACLE_H
#define ZTM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* mesh parameter block: nx, ny, nz, x0, y0, z_top, dx, dy, dz */
/* imesh parameter block: nx, ny, x0, y0, dx, dy, z_base */

void ora_pointmass_tfm(int di, int dj, int dk, int fh, int fv, int bfr,
                       const double* drho, const int* nn, long n_nn,
                       const double* surf, double* G, int nthreads);
void ora_pointmass_tfm_range(int di, int dj, int dk, int fh, int fv, int bfr,
                             const double* drho, const int* nn, long n_nn,
                             const double* surf, double* G, long s_lo, long s_hi,
                             int nthreads);
void ora_pointmass_adjoint(int di, int dj, int dk, int fh, int fv, int bfr, const int* nn,
                           long n_nn, const double* surf, const double* w, double* g,
                           int nthreads);
void ora_pointmass_gf(int bfr, int di, int dj, int dk, int fh, int fv,
                      const float* rho, long nthreads_total, const float* s,
                      float* g);
double ora_phi(double x, double y, double z);
long double ora_phil(long double x, long double y, long double z);
double ora_prism_unit(double xs, double ys, double zs, double x0, double x1,
                      double y0, double y1, double z0, double z1);
long double ora_prism_unitl(long double xs, long double ys, long double zs,
                            long double x0, long double x1, long double y0,
                            long double y1, long double z0, long double z1);
double ora_face_unit(double xs, double ys, double zs, double x0, double x1,
                     double y0, double y1, double zf);
void ora_prism_mesh(const double* mp, const double* rho, int ns,
                    const double* sxyz, double G, double* gz, int nthreads,
                    int use_long_double);
void ora_prism_list(long np, const double* geom, const double* rho, int ns,
                    const double* sxyz, double G, double* gz, int nthreads);
void ora_mesh_adjoint(const double* mp, int ns, const double* sxyz,
                      const double* resid, double G, double* g_rho,
                      int nthreads);
void ora_interface_fwd(const double* imp, const double* depth,
                       const double* rho_col, int ns, const double* sxyz,
                       double G, double* gz, int nthreads);
void ora_interface_adj(const double* imp, const double* depth,
                       const double* rho_col, int ns, const double* sxyz,
                       const double* resid, double G, double* g_rho,
                       double* g_depth, int nthreads);

/* density builder (TFM.cpp:85-89); rc is TFM's RC (TFM.cpp:218) */
void ora_density_geo(const double* rc, double* geo16);
void ora_density_tfm(int di, int dj, int dk, int fh, int fv, double vm, double ro, double dr,
                     const double* rc, const double* sea, const double* M, const double* v,
                     double* drho, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
