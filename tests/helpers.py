"""Shared inputs and error measures for the parity tests."""
import numpy as np


def rel_err(a, ref):
    """Normwise relative error max|a-ref| / max|ref| (the tolerance measure
    used throughout: per-station relative error is meaningless where the
    field crosses zero)."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.max(np.abs(ref))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - ref)) / scale)


def tfm_like_inputs(di, dj, dk, fh=1, fv=2, seed=0, sparsity=0.3):
    """drho on the fine grid, zero outside a selected set (as TFM.cpp:89
    leaves it), and station heights surf near the top of the grid."""
    rng = np.random.default_rng(seed)
    ii = (di - 1) * fh + 1
    jj = (dj - 1) * fh + 1
    kk = (dk - 1) * fv + 1
    drho = rng.normal(0.0, 0.1, ii * jj * kk)
    drho[rng.random(drho.size) < sparsity] = 0.0
    drho[np.abs(drho) <= 0.001] = 0.0
    surf = (dk - 3) + 0.37 + 0.2 * rng.random(di * dj)
    # TFM.cpp:89 keeps only nodes deeper than 10 km (one grid unit at
    # h = 10 km) below the surface; masses never sit next to a station
    k = (np.arange(ii * jj * kk) // (ii * jj)) / fv
    drho[k > surf.min() - 1.0] = 0.0
    return drho, surf


def small_mesh(nx=12, ny=10, nz=6, seed=0, dx=1000.0, dy=800.0, dz=500.0):
    import ztm_gb300
    rng = np.random.default_rng(seed)
    mesh = ztm_gb300.make_mesh(nx, ny, nz, dx, dy, dz, x0=-3000.0, y0=1500.0, z_top=200.0)
    rho = rng.normal(0.0, 200.0, nx * ny * nz)
    rho[rng.random(rho.size) < 0.1] = 0.0
    return mesh, rho


def awkward_stations(mesh, n_random=40, seed=1):
    """Random stations plus stations on faces, edges and vertices of the
    mesh, inside it, and outside it."""
    rng = np.random.default_rng(seed)
    x0, y0, zt = mesh.x0, mesh.y0, mesh.z_top
    X1 = x0 + mesh.nx * mesh.dx
    Y1 = y0 + mesh.ny * mesh.dy
    Zb = zt - mesh.nz * mesh.dz
    st = [
        (x0, y0, zt),                       # mesh vertex
        (x0 + mesh.dx, y0 + 2 * mesh.dy, zt),  # interior vertex on the top face
        (x0 + 0.5 * mesh.dx, y0 + 0.5 * mesh.dy, zt),  # top-face centre
        (x0 + 2 * mesh.dx, y0 + 0.3 * mesh.dy, zt + 50.0),  # above an edge
        (X1 + 3000.0, Y1 + 100.0, zt + 10.0),  # outside
        (0.5 * (x0 + X1), 0.5 * (y0 + Y1), 0.5 * (zt + Zb) + 0.25 * mesh.dz),  # inside
        (x0 - 500.0, y0 + mesh.dy, zt - mesh.dz),  # beside, on a layer plane
        # below the bottom, at the centre of the first padding layer under a
        # column centre (nz not a multiple of 8), and far below
        (x0 + 1.5 * mesh.dx, y0 + 0.5 * mesh.dy, Zb - 0.5 * mesh.dz),
        (x0 + 0.7 * mesh.dx, y0 + 1.2 * mesh.dy, Zb - 20.0 * mesh.dz),
    ]
    xs = rng.uniform(x0 - 2000.0, X1 + 2000.0, n_random)
    ys = rng.uniform(y0 - 2000.0, Y1 + 2000.0, n_random)
    zs = rng.uniform(zt + 1.0, zt + 3000.0, n_random)
    st += list(zip(xs, ys, zs))
    return np.array(st, dtype=np.float64)


def tfm_density_inputs(di=61, dj=61, dk=33, seed=0):
    """Synthetic inputs of the density builder shaped like TFM's: RC as
    TFM.cpp:218 builds it (h = 10 km), sea level near the top of the grid,
    a Moho about 35 km below it with relief, and a velocity field around
    the mantle velocity (crust slower)."""
    rng = np.random.default_rng(seed)
    h = 10.0
    rc = [-15.25, -72.5, (dk - 3) * h / 2 - 5, (di - 1) * h / 2, (dj - 1) * h / 2,
          (dk - 1) * h / 2, h, float(di), float(dj), float(dk)]
    X, Y = np.meshgrid(np.arange(di), np.arange(dj), indexing="xy")
    sea = (dk - 3) - 0.02 * ((X - di / 2) ** 2 + (Y - dj / 2) ** 2) / di + 0.05 * rng.random((dj, di))
    M = sea - 3.5 + 0.8 * np.sin(X / 7.0) * np.cos(Y / 5.0) + 0.1 * rng.random((dj, di))
    v = 8.0 + 0.3 * rng.standard_normal((dk, dj, di))
    return rc, sea.ravel(), M.ravel(), v.ravel()
