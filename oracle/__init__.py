"""CPU oracle of the gravity path - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package, and only to check results against (or as the timed
CPU baseline).
The product library never calls it; there is no CPU fallback.

Contents (oracle.c):
  pointmass_tfm   restatement of TFM.cpp:95-99 (double)
  pointmass_gf    restatement of GFM_GPU.cu:16-22 (float)
  prism_* / face  published closed form (no reference implementation)
  ref_gf          the reference GF kernel itself (compiled unchanged into
                  oracle/_ref/gf_ref.cubin) run on a GPU through the driver API
  ref_tfm         the reference's CPU gravity lambda itself (TFM.cpp:95-99 cut
                  verbatim out of TFM.cpp into oracle/_ref/tfm_gfm.cpp and
                  compiled with g++), all interior rows or a range of rows
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None
_runner = None
_tfm = None
_lm = None
NTHREADS = max(1, os.cpu_count() or 1)


def _load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        D = ctypes.c_double
        P = ctypes.c_void_p
        I = ctypes.c_int
        L = ctypes.c_long
        lib.ora_pointmass_tfm.argtypes = [I, I, I, I, I, I, P, P, L, P, P, I]
        lib.ora_pointmass_tfm_range.argtypes = [I, I, I, I, I, I, P, P, L, P, P, L, L, I]
        lib.ora_pointmass_gf.argtypes = [I, I, I, I, I, I, P, L, P, P]
        lib.ora_pointmass_adjoint.argtypes = [I, I, I, I, I, I, P, L, P, P, P, I]
        lib.ora_phi.argtypes = [D, D, D]
        lib.ora_phi.restype = D
        lib.ora_prism_unit.argtypes = [D] * 9
        lib.ora_prism_unit.restype = D
        lib.ora_face_unit.argtypes = [D] * 8
        lib.ora_face_unit.restype = D
        lib.ora_prism_mesh.argtypes = [P, P, I, P, D, P, I, I]
        lib.ora_prism_list.argtypes = [L, P, P, I, P, D, P, I]
        lib.ora_mesh_adjoint.argtypes = [P, I, P, P, D, P, I]
        lib.ora_interface_fwd.argtypes = [P, P, P, I, P, D, P, I]
        lib.ora_interface_adj.argtypes = [P, P, P, I, P, P, D, P, P, I]
        lib.ora_density_tfm.argtypes = [I, I, I, I, I, D, D, D, P, P, P, P, P, I]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def mesh_params(mesh):
    return np.array([mesh.nx, mesh.ny, mesh.nz, mesh.x0, mesh.y0, mesh.z_top,
                     mesh.dx, mesh.dy, mesh.dz], dtype=np.float64)


def imesh_params(im):
    return np.array([im.nx, im.ny, im.x0, im.y0, im.dx, im.dy, im.z_base], dtype=np.float64)


def pointmass_tfm(grid, drho, surf, nn=None, nthreads=None):
    """TFM.cpp:95-99.  nn defaults to the nodes with |drho| > grid.threshold
    (the list TFM.cpp:89 builds).  Returns G (di*dj); non-interior 0."""
    lib = _load()
    drho = _f64(drho)
    surf = _f64(surf)
    if nn is None:
        nn = np.nonzero(np.abs(drho) > grid.threshold)[0]
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    G = np.zeros(grid.di * grid.dj)
    lib.ora_pointmass_tfm(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, grid.bfr, _p(drho), _p(nn),
                          nn.size, _p(surf), _p(G), nthreads or NTHREADS)
    return G * grid.scale if grid.scale != 1.0 else G


def pointmass_tfm_sample(grid, drho, surf, s_lo, s_hi, nn=None, nthreads=None):
    """TFM.cpp:95-99 for interior stations s_lo..s_hi only (a bounded
    sample for timing).  Returns G (di*dj) with the sampled entries set."""
    lib = _load()
    drho = _f64(drho)
    surf = _f64(surf)
    if nn is None:
        nn = np.nonzero(np.abs(drho) > grid.threshold)[0]
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    G = np.zeros(grid.di * grid.dj)
    lib.ora_pointmass_tfm_range(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, grid.bfr, _p(drho),
                                _p(nn), nn.size, _p(surf), _p(G), s_lo, s_hi,
                                nthreads or NTHREADS)
    return G, nn.size


def pointmass_adjoint(grid, surf, w, nn=None, drho=None, nthreads=None):
    """Transpose of TFM.cpp:96-98 (grid units, times grid.scale like the
    forward): g[n] = sum over interior stations m of w[m] * dG[m]/d drho[n]
    for the nodes of nn (with multiplicity), or of |drho| > threshold when
    nn is None and drho is given, or every node."""
    lib = _load()
    surf = _f64(surf)
    w = _f64(w)
    ii = (grid.di - 1) * grid.fh + 1
    jj = (grid.dj - 1) * grid.fh + 1
    kk = (grid.dk - 1) * grid.fv + 1
    N = ii * jj * kk
    if nn is None:
        nn = np.nonzero(np.abs(_f64(drho)) > grid.threshold)[0] if drho is not None else np.arange(N)
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    g = np.zeros(N)
    lib.ora_pointmass_adjoint(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, grid.bfr, _p(nn), nn.size,
                              _p(surf), _p(w), _p(g), nthreads or NTHREADS)
    return g * grid.scale if grid.scale != 1.0 else g


def pointmass_gf(grid, rho32, s32, nthreads_total=None):
    """GFM_GPU.cu:16-22 in float, summed in thread order."""
    lib = _load()
    rho32 = np.ascontiguousarray(rho32, dtype=np.float32)
    s32 = np.ascontiguousarray(s32, dtype=np.float32)
    ii = (grid.di - 1) * grid.fh + 1
    n = nthreads_total if nthreads_total is not None else (rho32.size // ii) * ii
    g = np.zeros(grid.di * grid.dj, dtype=np.float32)
    lib.ora_pointmass_gf(grid.bfr, grid.di, grid.dj, grid.dk, grid.fh, grid.fv, _p(rho32), n,
                         _p(s32), _p(g))
    return g


def phi(x, y, z):
    return _load().ora_phi(x, y, z)


def prism_unit(xs, ys, zs, x0, x1, y0, y1, z0, z1):
    return _load().ora_prism_unit(xs, ys, zs, x0, x1, y0, y1, z0, z1)


def face_unit(xs, ys, zs, x0, x1, y0, y1, zf):
    return _load().ora_face_unit(xs, ys, zs, x0, x1, y0, y1, zf)


def prism_mesh(mesh, rho, stations, G=6.67e-11, nthreads=None, long_double=False):
    lib = _load()
    mp = mesh_params(mesh)
    rho = _f64(rho)
    st = _f64(stations).reshape(-1, 3)
    gz = np.zeros(st.shape[0])
    lib.ora_prism_mesh(_p(mp), _p(rho), st.shape[0], _p(st), G, _p(gz), nthreads or NTHREADS,
                       1 if long_double else 0)
    return gz


def prism_list(geom, rho, stations, G=6.67e-11, nthreads=None):
    lib = _load()
    geom = _f64(geom).reshape(-1, 6)
    rho = _f64(rho)
    st = _f64(stations).reshape(-1, 3)
    gz = np.zeros(st.shape[0])
    lib.ora_prism_list(geom.shape[0], _p(geom), _p(rho), st.shape[0], _p(st), G, _p(gz),
                       nthreads or NTHREADS)
    return gz


def mesh_adjoint(mesh, stations, resid, G=6.67e-11, nthreads=None):
    lib = _load()
    mp = mesh_params(mesh)
    st = _f64(stations).reshape(-1, 3)
    res = _f64(resid)
    g = np.zeros(mesh.nx * mesh.ny * mesh.nz)
    lib.ora_mesh_adjoint(_p(mp), st.shape[0], _p(st), _p(res), G, _p(g), nthreads or NTHREADS)
    return g


def interface_fwd(imesh, depth, rho_col, stations, G=6.67e-11, nthreads=None):
    lib = _load()
    ip = imesh_params(imesh)
    depth = _f64(depth)
    rho_col = _f64(rho_col)
    st = _f64(stations).reshape(-1, 3)
    gz = np.zeros(st.shape[0])
    lib.ora_interface_fwd(_p(ip), _p(depth), _p(rho_col), st.shape[0], _p(st), G, _p(gz),
                          nthreads or NTHREADS)
    return gz


def interface_adj(imesh, depth, rho_col, stations, resid, G=6.67e-11, nthreads=None):
    lib = _load()
    ip = imesh_params(imesh)
    depth = _f64(depth)
    rho_col = _f64(rho_col)
    st = _f64(stations).reshape(-1, 3)
    res = _f64(resid)
    nc = imesh.nx * imesh.ny
    gr = np.zeros(nc)
    gd = np.zeros(nc)
    lib.ora_interface_adj(_p(ip), _p(depth), _p(rho_col), st.shape[0], _p(st), _p(res), G,
                          _p(gr), _p(gd), nthreads or NTHREADS)
    return gr, gd


def density_tfm(di, dj, dk, fh, fv, vm, ro, dr, rc, sea, M, v, nthreads=None):
    """TFM.cpp:85-89: the fine-grid density perturbation drho."""
    lib = _load()
    rc = _f64(rc)
    sea, M, v = _f64(sea), _f64(M), _f64(v)
    N = ((di - 1) * fh + 1) * ((dj - 1) * fh + 1) * ((dk - 1) * fv + 1)
    out = np.zeros(N)
    lib.ora_density_tfm(di, dj, dk, fh, fv, vm, ro, dr, _p(rc), _p(sea), _p(M), _p(v), _p(out),
                        nthreads or NTHREADS)
    return out


# ---- the reference GF kernel itself (GPU host only) ----------------------
def ref_gf_available():
    return os.path.exists(_build.CUBIN) and os.path.exists(_build.RUNNER)


def ref_gf(grid, rho32, s32, reps=1):
    """Runs the unchanged reference GF kernel; returns (g float32, ms)."""
    global _runner
    if _runner is None:
        _build.build()
        r = ctypes.CDLL(_build.RUNNER)
        P = ctypes.c_void_p
        I = ctypes.c_int
        r.ref_gf_run.argtypes = [ctypes.c_char_p, I, I, I, I, I, I, P, ctypes.c_longlong, P, P, I,
                                 ctypes.POINTER(ctypes.c_float)]
        r.ref_gf_run.restype = I
        _runner = r
    rho32 = np.ascontiguousarray(rho32, dtype=np.float32)
    s32 = np.ascontiguousarray(s32, dtype=np.float32)
    g = np.zeros(grid.di * grid.dj, dtype=np.float32)
    ms = ctypes.c_float(0)
    rc = _runner.ref_gf_run(_build.CUBIN.encode(), grid.bfr, grid.di, grid.dj, grid.dk, grid.fh,
                            grid.fv, _p(rho32), rho32.size, _p(s32), _p(g), reps,
                            ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("reference GF run failed with code %d" % rc)
    return g, ms.value


# ---- the reference's CPU lambda itself (TFM.cpp:95-99) -------------------
def ref_tfm_available():
    _build.build()
    return os.path.exists(_build.TFM_LIB)


def _tfm_lib():
    global _tfm
    if _tfm is None:
        if not ref_tfm_available():
            raise RuntimeError("oracle/_ref/libref_tfm.so is not built (no reference TFM.cpp and "
                               "no generated harness)")
        t = ctypes.CDLL(_build.TFM_LIB)
        P = ctypes.c_void_p
        I = ctypes.c_int
        LL = ctypes.c_longlong
        t.ref_tfm_gfm.argtypes = [I, I, I, I, I, I, P, LL, P, LL, P, P]
        t.ref_tfm_gfm.restype = None
        t.ref_tfm_gfm_rows.argtypes = [I, I, I, I, I, I, P, LL, P, LL, P, P, I, I]
        t.ref_tfm_gfm_rows.restype = None
        _tfm = t
    return _tfm


def _tfm_args(grid, drho, surf, nn):
    drho = _f64(drho)
    surf = _f64(surf)
    if nn is None:
        nn = np.nonzero(np.abs(drho) > grid.threshold)[0]
    nn = np.ascontiguousarray(nn, dtype=np.int32)
    return drho, surf, nn


def ref_tfm(grid, drho, surf, nn=None):
    """G (di*dj) from the reference's own compiled lambda, every interior
    row on its own thread, as TFM.cpp:99 launches it; non-interior 0."""
    t = _tfm_lib()
    drho, surf, nn = _tfm_args(grid, drho, surf, nn)
    G = np.zeros(grid.di * grid.dj)
    t.ref_tfm_gfm(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, grid.bfr, _p(drho), drho.size,
                  _p(nn), nn.size, _p(surf), _p(G))
    return G * grid.scale if grid.scale != 1.0 else G


def ref_tfm_rows(grid, drho, surf, row_lo, row_hi, nn=None):
    """The reference lambda on station rows j0 in [row_lo, row_hi) only (one
    thread per row); returns (G, nodes summed).  Unscaled (grid units)."""
    t = _tfm_lib()
    drho, surf, nn = _tfm_args(grid, drho, surf, nn)
    G = np.zeros(grid.di * grid.dj)
    t.ref_tfm_gfm_rows(grid.di, grid.dj, grid.dk, grid.fh, grid.fv, grid.bfr, _p(drho), drho.size,
                       _p(nn), nn.size, _p(surf), _p(G), int(row_lo), int(row_hi))
    return G, nn.size


# ---- the reference's own LM step (zmath.cpp + TFM.cpp:159-160) -----------
def ref_lm_available():
    _build.build()
    return os.path.exists(_build.LM_LIB)


def ref_lm_steps(J, r, b, sig, damping):
    """B (nd x ncols) and JJ from the reference's zmath.cpp (MTM, inv, T and
    its operators, compiled unchanged) and the two statements of LMA::fit
    (TFM.cpp:159-160)."""
    global _lm
    if _lm is None:
        if not ref_lm_available():
            raise RuntimeError("oracle/_ref/libref_lm.so is not built")
        t = ctypes.CDLL(_build.LM_LIB)
        P = ctypes.c_void_p
        I = ctypes.c_int
        t.ref_lm_steps.argtypes = [P, I, I, P, P, P, P, I, P, P]
        t.ref_lm_steps.restype = None
        _lm = t
    J = _f64(J)
    nrows, ncols = J.shape
    r, b, sig = _f64(r), _f64(b), _f64(sig)
    dm = _f64(damping).reshape(-1, 2)
    B = np.zeros((dm.shape[0], ncols))
    JJ = np.zeros((ncols, ncols))
    _lm.ref_lm_steps(_p(J), nrows, ncols, _p(r), _p(b), _p(sig), _p(dm), dm.shape[0], _p(B), _p(JJ))
    return B, JJ


def lm_steps(J, r, b, sig, damping):
    """TFM.cpp:159-160 restated in numpy (when the reference sources are
    absent): JJ = J^T J, B[d] = b + inv(JJ + d0 diag(JJ) + d1 diag(1/sig^2)) J^T r."""
    J = _f64(J)
    JJ = J.T @ J
    g = J.T @ _f64(r)
    out = []
    for d0, d1 in _f64(damping).reshape(-1, 2):
        A = JJ + d0 * np.diag(np.diag(JJ)) + d1 * np.diag(1.0 / _f64(sig) ** 2)
        out.append(_f64(b) + np.linalg.inv(A) @ g)
    return np.array(out), JJ
