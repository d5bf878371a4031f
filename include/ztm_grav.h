/*
 * ztm_grav.h - C ABI of the GB300 gravity forward model and adjoint.
 *
 * This is the in-process boundary that replaces the gravity section of ZTM's
 * forward model:
 *   - TFM.cpp:90-94  GPU branch: float32 files in /dev/shm plus popen("./GFM")
 *   - TFM.cpp:95-99  CPU branch: std::thread lambda, point-mass sum in double
 *   - GFM_GPU.cu:16-34  the GF kernel and its host main()
 * The caller (the C++ inversion driver) owns every host array; the library
 * copies in and out, or, with ZTM_FLAG_DEVICE_PTRS, reads and writes device
 * pointers in place.  A context owns its device buffers and CUDA stream.
 * No function throws; every entry point returns an int status (0 = ok) and
 * ztm_last_error() gives the message.  A non-zero status is the signal on
 * which the caller falls back to its CPU path, exactly as TFM.cpp:95 does when
 * the GPU model did not compile (TFM.cpp:207-208).
 *
 * Threading: one context per host thread, or serialise calls on a context.
 * The library keeps no global CUDA state besides the device it was created on.
 *
 * Units.  Point-mass mode keeps the reference's grid units (indices, k up,
 * density in g/cc, gz in mGal with the 66.7 constant of TFM.cpp:98).  Prism
 * and interface modes use metres (z up), kg/m^3 and mGal; gz is the downward
 * attraction (positive above excess mass), the sign convention of TFM.cpp:98.
 */
#ifndef ZTM_GRAV_H
#define ZTM_GRAV_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  ZTM_OK = 0,
  ZTM_ERR_ARG = -1,     /* bad dimensions, null pointers, bad flags */
  ZTM_ERR_ALLOC = -2,   /* device or pinned-host allocation failed */
  ZTM_ERR_CUDA = -3,    /* a CUDA runtime call or kernel launch failed */
  ZTM_ERR_TIMEOUT = -4, /* a bounded device-side wait gave up */
  ZTM_ERR_NODEV = -5,   /* no CUDA device, or the device id is invalid */
  ZTM_ERR_RANGE = -6    /* a size exceeds a documented limit */
};

/* ---- precision / method ----------------------------------------------- */
enum {
  ZTM_PREC_FP64 = 0,  /* plain: every pair in double (closed form / pow) */
  ZTM_PREC_FP32 = 1,  /* every pair in float with compensated sums */
  ZTM_PREC_MIXED = 2  /* prism modes: far pairs in float (moment expansion
                         to sixth order on 3-D meshes, horizontal expansion
                         to fourth order for interface columns; compensated
                         sums), near pairs and the final per-station sums in
                         double */
};

/* ---- flags ----------------------------------------------------------- */
enum {
  ZTM_FLAG_DEVICE_PTRS = 1, /* all array arguments are device pointers */
  ZTM_FLAG_AUTOTUNE = 2     /* prism forward and batch: on the first call
                               for these shapes (mesh and station counts;
                               for a batch, every job's), time the candidate
                               launch shapes (forward: columns per stage x
                               items per block; batch: stage size x pairs
                               per item) and keep the fastest on the context */
};

typedef struct ztm_ctx ztm_ctx;

/* Reference grid of the point-mass model (TFM.cpp:83 and GFM_GPU.cu:24).
 * Fine grid: ii=(di-1)*fh+1, jj=(dj-1)*fh+1, kk=(dk-1)*fv+1 nodes, flat index
 * n = i + j*ii + k*ii*jj.  Stations: the di*dj coarse nodes with
 * bfr <= i0 < di-bfr and bfr <= j0 < dj-bfr, at height surf[i0+j0*di]. */
typedef struct {
  int di, dj, dk;   /* coarse grid dimensions */
  int fh, fv;       /* horizontal / vertical refinement */
  int bfr;          /* boundary buffer without stations */
  double threshold; /* nodes with |drho| > threshold contribute (0.001) */
  double scale;     /* result multiplier: h/10 for spacing h km (1.0) */
} ztm_grid;

/* Regular prism mesh: nx*ny columns of nz layers, layer 0 at the top.
 * Prism (ix,iy,l) spans [x0+ix*dx, x0+(ix+1)*dx] x [y0+iy*dy, ...] x
 * [z_top-(l+1)*dz, z_top-l*dz].  Density index: ix + nx*(iy + ny*l). */
typedef struct {
  int nx, ny, nz;
  double x0, y0, z_top;
  double dx, dy, dz;
} ztm_mesh;

/* Interface mesh: nx*ny prism columns.  Column (ix,iy) spans the cell
 * horizontally and z in [z_base, -depth[ix+nx*iy]] (depth > 0 below z=0). */
typedef struct {
  int nx, ny;
  double x0, y0;
  double dx, dy;
  double z_base; /* elevation of the column bases, e.g. -45000 */
} ztm_imesh;

/* Per-call options.  Zero-initialise and set what you need. */
typedef struct {
  int precision;  /* ZTM_PREC_* */
  int flags;      /* ZTM_FLAG_* */
  double G;       /* gravitational constant; 0 selects 6.67e-11, the value
                     that TFM.cpp:98's 66.7 mGal factor bakes in */
  double near_q;  /* mixed mode: pairs closer than near_q prism half-
                     diagonals are evaluated in double; 0 selects 4 for
                     the regular 3-D mesh (sixth-order far field), 6 for
                     the explicit prism list and the interface columns */
  int tile;       /* reserved, 0 */
  int chunk;      /* prism columns per block; 0 = chosen by the library
                     (from the autotuner's cache when ZTM_FLAG_AUTOTUNE) */
} ztm_opts;

/* One job of a batched launch: nmodels density models that share one
 * geometry and one station set.  rho is nmodels x (nx*ny*nz), gz is
 * nmodels x ns, model-major. */
typedef struct {
  ztm_mesh mesh;
  int nmodels;
  const double* rho;
  int ns;
  const double* sxyz;
  double* gz;
} ztm_job;

/* ---- context --------------------------------------------------------- */
int ztm_version(void);
/* Creates a context on CUDA device `device` with its own non-blocking
 * stream.  Replaces the per-call context creation of GFM_GPU.cu:28-30. */
int ztm_ctx_create(int device, ztm_ctx** out);
void ztm_ctx_destroy(ztm_ctx* ctx);
/* Message of the last failed call on this context ("" if none). */
const char* ztm_last_error(const ztm_ctx* ctx);
/* Use `stream` (a cudaStream_t) for subsequent calls; NULL restores the
 * context's own stream.  The caller keeps ownership of the stream. */
int ztm_ctx_set_stream(ztm_ctx* ctx, void* stream);
void* ztm_ctx_stream(ztm_ctx* ctx);
/* Number of kernels this context has launched so far. */
long long ztm_ctx_launches(const ztm_ctx* ctx);
/* Waits for the context's stream and reports device-side errors of calls
 * made with ZTM_FLAG_DEVICE_PTRS (those calls return without waiting). */
int ztm_ctx_sync(ztm_ctx* ctx);

/* ---- tracing ----------------------------------------------------------- */
/* While enabled, the context brackets each of its compute kernels with CUDA
 * events on its stream.  ztm_ctx_profile_read waits for the stream, returns
 * the summed device time (ms) and launch count of the kernels whose name
 * contains `name` ("" = all), and clears the records.  Kernel names:
 * pointmass, prism_far (the mixed forward's far fields and near regions),
 * prism_f64, prism_list, adjoint_far (the mixed adjoint's far fields and
 * near regions), adjoint_f64, iface_far, iface_near, iface_f64, batch,
 * density.
 * The reference's only timer is a host clock (zmath.cpp:265-268). */
int ztm_ctx_profile(ztm_ctx* ctx, int enable);
int ztm_ctx_profile_read(ztm_ctx* ctx, const char* name, double* ms,
                         long long* count);
/* The autotuner's record: the candidates it timed since the context was
 * created (ZTM_FLAG_AUTOTUNE), four ints each -- for a batched launch (stage
 * KB per model group, or for the tensor-core variant 4 the 16-layer blocks
 * per accumulator read-back; log2 of the pairs per far item; kernel variant;
 * microseconds); writes at most max_rows rows and returns how many it wrote
 * (negative on a bad argument). */
int ztm_ctx_tuning(const ztm_ctx* ctx, int* rows, int max_rows);
/* Form counters of the mixed prism forward.  While enabled, the forward runs
 * a counting variant of its far kernel (the same arithmetic plus one counter
 * update per column and thread) that adds up the (station, prism) slots it
 * evaluates in each form of the far-field expansion.  ztm_ctx_form_counts
 * waits for the stream and returns, then clears: counts[0] slots in the
 * sixth-order form, [1] second order, [2] second order by column pairs
 * (slots include the near-region layers a masked group evaluates and drops,
 * and the padding of nz to a multiple of 8), [3] closed-form corner-function
 * evaluations (Phi) of the near regions.  These are the numerators of the
 * executed-flop roofline; the reference has no counterpart. */
int ztm_ctx_count_forms(ztm_ctx* ctx, int enable);
int ztm_ctx_form_counts(ztm_ctx* ctx, long long* counts);
/* Test hook of the timeout path (no GPU fault involved).  With polls > 0,
 * every copy-arrival wait of the mixed prism forward's far kernel, and of the
 * tensor-core far items of the batched launch, waits instead on a barrier
 * that nothing completes and gives up after `polls` tests; each block then
 * records a timeout, waits (with the full bound) for the copies and MMAs it
 * has in flight, frees its tensor memory and stops, and the call returns
 * ZTM_ERR_TIMEOUT.  polls = 0 switches the hook off; the context stays
 * usable throughout. */
int ztm_ctx_test_timeout(ztm_ctx* ctx, unsigned int polls);
/* Issue-rate micro-benchmarks of the device, the denominators of the
 * compute roofline: kind 0 = FP32 FMA (TFLOP/s, 2 flops per FMA), 1 = FP64
 * FMA (TFLOP/s), 2 = float rsqrt on the special-function unit (Gop/s). */
int ztm_measure_peak(ztm_ctx* ctx, int kind, double* value);

/* ---- point-mass mode (reference model) ------------------------------- */
/* Replaces TFM.cpp:90-99 and GFM_GPU.cu:16-34.  drho has ii*jj*kk values
 * (g/cc), surf di*dj station heights (grid units), G receives di*dj values
 * in mGal: interior stations get the sum, the rest are set to 0 (as the GPU
 * branch returns them, TFM.cpp:94).  If nn is non-NULL only the n_nn listed
 * nodes contribute (the CPU branch's list, TFM.cpp:89,97; a node listed
 * twice counts twice, as in that loop); otherwise nodes with
 * |drho| > grid->threshold.  An nn entry outside the grid fails the call
 * (ZTM_ERR_RANGE; with device pointers it is skipped on the device and
 * reported at the call's end).  precision: ZTM_PREC_FP64 or _FP32. */
int ztm_gfm_pointmass(ztm_ctx* ctx, const ztm_grid* grid, const double* drho,
                      const int* nn, long long n_nn, const double* surf,
                      double* G, int precision, int flags);

/* Adjoint (transposed sum) of ztm_gfm_pointmass: for every fine-grid node
 * n, g_drho[n] = sum over interior stations m of w[m] * dG[m]/d drho[n]
 *             = scale * 66.7/(fh^2 fv) * sum_m w[m] (k0_m - k_n) / r_mn^3,
 * i.e. J^T w for the station weights w (di*dj values; the interior ones are
 * read).  Node selection, as in the forward: with nn, only the listed nodes
 * (times their multiplicity; 0 elsewhere); else, with drho, the nodes with
 * |drho| > grid->threshold; with neither, every node.  No counterpart in the
 * reference: its optimiser builds these derivatives by finite differences of
 * whole forward runs (TFM.cpp:124-135).  precision: ZTM_PREC_FP64 or _FP32. */
int ztm_gfm_pointmass_adjoint(ztm_ctx* ctx, const ztm_grid* grid, const double* drho,
                              const int* nn, long long n_nn, const double* surf,
                              const double* w, double* g_drho, int precision, int flags);

/* The gravity part of the reference misfit, TFM.cpp:101-103, with its
 * gradient: G = the point-mass forward (as ztm_gfm_pointmass, same node
 * selection), res[t] = GD[m]/gsig - (G[m] + g0)/gsig over the bfr interior
 * in TFM's order (i0 outer, j0 inner: t = (i0-bfr)*(dj-2bfr) + (j0-bfr)),
 * *ssq = sum res^2 (the gravity terms of FM::ssq), and, if asked for,
 * g_drho = d ssq / d drho (N values, by the adjoint above) and
 * *g_g0 = d ssq / d g0.  res, G, g_drho, g_g0 may be NULL.  With
 * ZTM_FLAG_DEVICE_PTRS every array and ssq / g_g0 are device pointers. */
int ztm_gfm_pointmass_misfit(ztm_ctx* ctx, const ztm_grid* grid, const double* drho,
                             const int* nn, long long n_nn, const double* surf,
                             const double* GD, double g0, double gsig, double* ssq,
                             double* res, double* G, double* g_drho, double* g_g0,
                             int precision, int flags);

/* Allocation-free point-mass forward.  No counterpart in the reference.
 * For callers that cannot allocate device memory at the time of the call
 * (a host that fixes the GPU memory budget up front, work issued while a
 * stream is being captured, a real-time loop that must not allocate): the
 * same sum as ztm_gfm_pointmass with drho, surf and G as DEVICE pointers on
 * the current device, launched on `stream` (a cudaStream_t; NULL = the
 * legacy default stream) and not waited for.  No context, no staging, no
 * cudaMalloc/cudaFree: the scratch is a fixed 4 MiB array reserved in each
 * GPU that loads the library.  Limits: at most 524,256 interior stations
 * (ZTM_ERR_RANGE beyond); all nodes with |drho| > grid->threshold contribute
 * (no nn list).  It runs the full-grid gather (nodes in grid order), not the
 * node-column gather of ztm_gfm_pointmass, whose column layout needs a
 * workspace, so it is slower than that entry on large grids.  Every call on
 * a device shares that array, so calls that can overlap on one GPU race:
 * serialise them on one stream.  The first call on each device (and the
 * first after a cudaDeviceReset) looks the array up (cudaGetSymbolAddress);
 * make it before any stream capture starts.  A CUDA error already pending
 * when the call starts is left pending and reported as ZTM_ERR_CUDA.
 * Returns ZTM_OK, ZTM_ERR_ARG, ZTM_ERR_RANGE, ZTM_ERR_NODEV or
 * ZTM_ERR_CUDA. */
int ztm_gfm_pointmass_noalloc(const ztm_grid* grid, const double* drho,
                              const double* surf, double* G, int precision,
                              void* stream);

/* Density-perturbation builder of TFM.cpp:83-89 on the GPU.  vm, ro, dr are
 * the mantle velocity, the crust/mantle contrast as used in the loop
 * (TFM.cpp:84 negates the parameter) and the velocity-to-density ratio; rc
 * is TFM's RC vector (TFM.cpp:218: ref lat, lon, depth, origin x, y, z
 * offsets, spacing h, di, dj, dk).  sea, M (di*dj) and v (di*dj*dk) are the
 * reference's sea-level map, rendered Moho and velocity grids.  drho gets
 * the fine-grid perturbation, zero where TFM.cpp:89 leaves a node out of nn;
 * *n_selected (host mode only, else -1) the number of selected nodes. */
typedef struct {
  int di, dj, dk, fh, fv;
  double vm, ro, dr;
  double rc[10];
} ztm_density_params;
int ztm_density_build(ztm_ctx* ctx, const ztm_density_params* p,
                      const double* sea, const double* M, const double* v,
                      double* drho, long long* n_selected, int flags);
/* TFM.cpp:83-99 in one call: the density builder above followed by the
 * point-mass forward over the nodes it selects, with drho kept in device
 * memory between the two (no drho round trip through the host).  grid
 * supplies bfr, threshold and scale and must have the dims of p; surf and G
 * are as in ztm_gfm_pointmass.  With the reference's threshold 0.001 the
 * result equals ztm_density_build + ztm_gfm_pointmass with TFM's nn list. */
int ztm_gfm_pointmass_model(ztm_ctx* ctx, const ztm_density_params* p,
                            const ztm_grid* grid, const double* sea,
                            const double* M, const double* v,
                            const double* surf, double* G, int precision,
                            int flags);

/* TFM.cpp:83-103 with its gradient: the density builder, the point-mass
 * forward over the nodes it selects, the misfit of ztm_gfm_pointmass_misfit,
 * and, when any of g_M, g_v, g_par is non-NULL, one adjoint pass chained back
 * through the builder: g_M (di*dj) = d ssq / d M, g_v (di*dj*dk) =
 * d ssq / d v, g_par[0..3] = d ssq / d (vm, ro, dr, g0), with ro as the loop
 * uses it (TFM.cpp:84 takes ro = -B[...], so d ssq / d B = -g_par[1]).  The
 * builder's node selection is held fixed (the derivative a small finite-
 * difference step sees).  One forward and one adjoint replace the gravity
 * columns of the finite-difference Jacobian of TFM.cpp:124-135 (vm, ro, dr,
 * g0 and, through the rendered Moho M, the Moho nodes; the natural-neighbour
 * rendering of the nodes into M, NNI.cpp, stays with the caller). */
int ztm_gfm_pointmass_model_misfit(ztm_ctx* ctx, const ztm_density_params* p,
                                   const ztm_grid* grid, const double* sea, const double* M,
                                   const double* v, const double* surf, const double* GD,
                                   double g0, double gsig, double* ssq, double* res, double* G,
                                   double* g_M, double* g_v, double* g_par, int precision,
                                   int flags);

/* ---- prism mode -------------------------------------------------------- */
/* gz[s] = sum over all prisms of the closed-form attraction of prism p at
 * station s (sxyz is ns x 3: x, y, z).  No counterpart in the reference code
 * (it has only the point-mass model); it is the model the gravity path of
 * TFM.cpp:83-99 approximates. */
int ztm_gfm_prism(ztm_ctx* ctx, const ztm_mesh* mesh, const double* rho,
                  int ns, const double* sxyz, double* gz, const ztm_opts* opt);

/* Explicit prism list: geom is np x 6 (x0,x1,y0,y1,z0,z1), rho np values. */
int ztm_gfm_prism_list(ztm_ctx* ctx, long long np, const double* geom,
                       const double* rho, int ns, const double* sxyz,
                       double* gz, const ztm_opts* opt);

/* Adjoint of ztm_gfm_prism: g_rho[p] = sum_s resid[s] * dgz[s]/drho[p],
 * i.e. d(0.5*|gz-d|^2)/d(rho) for resid = gz-d.  Supersedes the gravity
 * columns of the finite-difference Jacobian (TFM.cpp:124-135). */
int ztm_gfm_adjoint(ztm_ctx* ctx, const ztm_mesh* mesh, int ns,
                    const double* sxyz, const double* resid, double* g_rho,
                    const ztm_opts* opt);

/* ---- interface mode ---------------------------------------------------- */
/* Forward of an interface mesh: column c has density rho_col[c] and its top
 * at depth[c] (m below z=0). */
int ztm_gfm_interface(ztm_ctx* ctx, const ztm_imesh* mesh,
                      const double* depth, const double* rho_col, int ns,
                      const double* sxyz, double* gz, const ztm_opts* opt);

/* Adjoint of ztm_gfm_interface: g_rho[c] = sum_s resid[s]*dgz[s]/drho[c]
 * and g_depth[c] = sum_s resid[s]*dgz[s]/ddepth[c] (analytic top-face
 * derivative).  Either output may be NULL. */
int ztm_gfm_interface_adjoint(ztm_ctx* ctx, const ztm_imesh* mesh,
                              const double* depth, const double* rho_col,
                              int ns, const double* sxyz, const double* resid,
                              double* g_rho, double* g_depth,
                              const ztm_opts* opt);

/* Directional derivative of the interface forward along a depth change
 * (Jacobian times vector, the forward-mode counterpart of g_depth):
 * dgz[s] = sum_c dgz[s]/ddepth[c] * d_depth[c] (mGal per metre of d_depth),
 * from the same top-face integral as the adjoint.  With the adjoint it gives
 * Gauss-Newton products J v and J^T w without forming J.  No counterpart in
 * the reference, whose optimiser builds J by finite differences of whole
 * forward runs (TFM.cpp:124-135). */
int ztm_gfm_interface_jvp(ztm_ctx* ctx, const ztm_imesh* mesh,
                          const double* depth, const double* rho_col,
                          const double* d_depth, int ns, const double* sxyz,
                          double* dgz, const ztm_opts* opt);

/* Forward + misfit + adjoint in one call: gz = F(depth, rho_col),
 * *misfit = 0.5*sum (gz-data)^2, gradients as ztm_gfm_interface_adjoint.
 * gz, g_rho, g_depth may be NULL. */
int ztm_gfm_interface_misfit(ztm_ctx* ctx, const ztm_imesh* mesh,
                             const double* depth, const double* rho_col,
                             int ns, const double* sxyz, const double* data,
                             double* misfit, double* gz, double* g_rho,
                             double* g_depth, const ztm_opts* opt);

/* Nonlinear inversion of the column tops: minimises
 *   0.5*|gz(depth) - data|^2 + 0.5*lambda*sum_neighbours (m_i - m_j)^2,
 * m = depth in km, by L-BFGS with an Armijo line search, one forward and one
 * adjoint (ztm_gfm_interface_misfit) per evaluation.  depth (m) is the
 * start model on entry and the result on return.  history (iterations+1
 * values, may be NULL) receives the data misfit 0.5*|r|^2 before each
 * iteration and at the end; *n_done the iterations taken.  Host arrays
 * only.  Replaces the damped Gauss-Newton loop of LMA::fit (TFM.cpp:155-167)
 * for the gravity interface, whose Jacobian came from finite differences. */
int ztm_invert_interface(ztm_ctx* ctx, const ztm_imesh* mesh, double* depth,
                         const double* rho_col, int ns, const double* sxyz,
                         const double* data, double lambda, int iterations,
                         const ztm_opts* opt, double* history, int* n_done);

/* The same inversion by Gauss-Newton: each iteration solves
 * (J^T J + lambda L) step = -gradient with at most cg_iterations conjugate-
 * gradient steps, each one ztm_gfm_interface_jvp (J v) and one depth adjoint
 * (J^T w), J never formed, then takes the projected step with a
 * backtracking line search.  Same objective, units, bounds, history and
 * n_done as ztm_invert_interface.  The reference's damped Gauss-Newton
 * (TFM.cpp:155-167) forms J^T J from a finite-difference Jacobian. */
int ztm_invert_interface_gn(ztm_ctx* ctx, const ztm_imesh* mesh, double* depth,
                            const double* rho_col, int ns, const double* sxyz,
                            const double* data, double lambda, int iterations,
                            int cg_iterations, const ztm_opts* opt, double* history,
                            int* n_done);

/* ---- damped Gauss-Newton step (normal equations) ------------------------ */
/* The trial models of one LMA::fit iteration (TFM.cpp:159-160): JJ = J^T J
 * (zmath.cpp:260-262 MTM), M = diag(diag(JJ)), A = diag(1/sig^2) and, for
 * each of the nd damping pairs (d0, d1) in `damping` (nd x 2),
 *   B[d] = b + inv(JJ + d0 M + d1 A) J^T r
 * (the reference inverts by Gauss-Jordan with partial pivoting,
 * zmath.cpp:129-140; here the system is factorised by blocked LU with the
 * same pivot rule and the right-hand side attached, which gives the same
 * step up to rounding).  J is nrows x ncols, row-major
 * (J[data][parameter], as Jac returns it), r the nrows residuals y - f, b and
 * sig ncols values, B nd x ncols; JJ (ncols x ncols) is returned if non-NULL.
 * A singular system leaves its B row equal to b, as the reference's inv
 * returns a zero matrix there.  Double precision throughout.  Limits:
 * ncols <= 32768 and nd*ncols*(ncols+1) < 2^31. */
int ztm_lm_steps(ztm_ctx* ctx, const double* J, int nrows, int ncols, const double* r,
                 const double* b, const double* sig, const double* damping, int nd,
                 double* B, double* JJ, int flags);

/* ---- batched ----------------------------------------------------------- */
/* Evaluates every job (trial models of a line search, independent regional
 * meshes of uneven size) in one persistent launch, replayed from a CUDA
 * graph cached on the context when the job shapes repeat.  Replaces the
 * sequential FM evaluations of the damping trials (TFM.cpp:165). */
int ztm_gfm_batch(ztm_ctx* ctx, const ztm_job* jobs, int njobs,
                  const ztm_opts* opt);

#ifdef __cplusplus
}
#endif
#endif /* ZTM_GRAV_H */
