"""Seeded synthetic meshes, densities and stations for the benchmark
workloads.  The reference's real inputs (WGM2012 Bouguer anomaly, ETOPO5
topography) are not available, so these stand in with the stated shapes,
sizes and value distributions.

Random fields: numpy PCG64(seed) white noise, FFT-filtered with a Gaussian
kernel whose standard deviation is half the correlation length, then
standardised.  Fractal topography: spectral synthesis with power
~ k^-(2H+2), rescaled to the stated range.
"""
import numpy as np

from .gfm import make_grid, make_imesh, make_mesh


def gaussian_field(shape, spacing, corr, rng):
    """Zero-mean, unit-std Gaussian random field on a regular grid."""
    noise = rng.standard_normal(shape)
    f = np.fft.rfftn(noise)
    ks = []
    for ax, (n, d) in enumerate(zip(shape, spacing)):
        k = np.fft.rfftfreq(n, d) if ax == len(shape) - 1 else np.fft.fftfreq(n, d)
        ks.append(2 * np.pi * k)
    grids = np.meshgrid(*ks, indexing="ij")
    k2 = sum(g * g for g in grids)
    sig = corr / 2.0
    f *= np.exp(-0.5 * k2 * sig * sig)
    out = np.fft.irfftn(f, s=shape, axes=tuple(range(len(shape))))
    out -= out.mean()
    sd = out.std()
    return out / sd if sd > 0 else out


def fractal_surface(n, spacing, H, rng):
    noise = rng.standard_normal((n, n))
    f = np.fft.rfft2(noise)
    kx = np.fft.fftfreq(n, spacing)[:, None]
    ky = np.fft.rfftfreq(n, spacing)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = np.inf
    f *= k ** (-(2 * H + 2) / 2.0)
    s = np.fft.irfft2(f, s=(n, n))
    return s


def _layer_major(field_xyz):
    """(nx, ny, nz) array -> flat density index ix + nx*(iy + ny*l)."""
    return np.ascontiguousarray(np.transpose(field_xyz, (2, 1, 0))).reshape(-1)


def plain_mesh_64x64x32(seed=1):
    """64x64x32 prisms of 2x2x1 km, top at z=0; density: Gaussian field,
    sigma 150 kg/m^3, correlation 8 km; 32x32 stations on a 4 km grid at
    z=+100 m, over the centres of the even columns."""
    rng = np.random.default_rng(seed)
    mesh = make_mesh(64, 64, 32, 2000.0, 2000.0, 1000.0)
    f = gaussian_field((64, 64, 32), (2000.0, 2000.0, 1000.0), 8000.0, rng) * 150.0
    rho = _layer_major(f)
    xs = 1000.0 + 4000.0 * np.arange(32)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    st = np.stack([X.ravel(), Y.ravel(), np.full(X.size, 100.0)], axis=1)
    return mesh, rho, st


def draped_mesh_256x256x64(seed=2, n_boxes=20):
    """256x256x64 prisms of 1x1x0.5 km, top at z=0; density: Gaussian field
    (correlation 5 km) scaled to max |rho| = 300 kg/m^3, plus 20 random box
    anomalies of +-300 kg/m^3; 128x128 stations over the even columns, draped
    on a fractal surface (H = 0.8) rescaled to 0..3 km."""
    rng = np.random.default_rng(seed)
    nx = ny = 256
    nz = 64
    mesh = make_mesh(nx, ny, nz, 1000.0, 1000.0, 500.0)
    f = gaussian_field((nx, ny, nz), (1000.0, 1000.0, 500.0), 5000.0, rng)
    f *= 300.0 / np.abs(f).max()
    for _ in range(n_boxes):
        sx, sy = rng.integers(2, 21, size=2)
        sz = rng.integers(2, 21)
        x0 = rng.integers(0, nx - sx)
        y0 = rng.integers(0, ny - sy)
        z0 = rng.integers(0, nz - sz)
        f[x0:x0 + sx, y0:y0 + sy, z0:z0 + sz] += rng.choice([-300.0, 300.0])
    rho = _layer_major(f)
    topo = fractal_surface(128, 2000.0, 0.8, rng)
    topo = (topo - topo.min()) / (topo.max() - topo.min()) * 3000.0
    xs = 500.0 + 2000.0 * np.arange(128)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    st = np.stack([X.ravel(), Y.ravel(), topo.T.ravel()], axis=1)
    return mesh, rho, st


def moho_columns(seed=3, n=256, ns_side=128, cell=1000.0, z_base=-45000.0, contrast=-400.0,
            noise_mgal=0.05):
    """Interface columns: n x n cells, bases at 45 km, tops on a smooth
    Moho-like surface between 20 and 45 km depth (Gaussian field, correlation
    40 km), contrast -400 kg/m^3; ns_side^2 stations at z=0 over the cell
    centres of a regular sub-grid.  Returns (imesh, depth_true, rho_col,
    stations, depth_start)."""
    rng = np.random.default_rng(seed)
    im = make_imesh(n, n, cell, cell, z_base)
    f = gaussian_field((n, n), (cell, cell), 40000.0, rng)
    depth = 20000.0 + (f - f.min()) / (f.max() - f.min()) * 25000.0
    depth = np.ascontiguousarray(depth.T).reshape(-1)  # index ix + n*iy
    rho = np.full(n * n, contrast)
    step = n // ns_side
    xs = (np.arange(ns_side) * step + 0.5 * step) * cell
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    st = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)
    start = np.full(n * n, float(depth.mean()))
    return im, depth, rho, st, start


def line_search_batch(seed=4, n_trials=32, n_regional=16):
    """Batched workload: 32 line-search trials m + alpha*p (alpha in [0,2])
    on the 256x256x64 draped mesh, and 16 regional meshes of uneven size
    (64^3 up to 192x192x48 prisms, 32^2 to 128^2 stations)."""
    rng = np.random.default_rng(seed)
    mesh, rho, st = draped_mesh_256x256x64()
    p = _layer_major(gaussian_field((256, 256, 64), (1000.0, 1000.0, 500.0), 10000.0, rng) * 30.0)
    alphas = np.linspace(0.0, 2.0, n_trials)
    trials = rho[None, :] + alphas[:, None] * p[None, :]
    jobs = [(mesh, trials, st)]
    for _ in range(n_regional):
        nx = int(rng.integers(64, 193))
        ny = int(rng.integers(64, 193))
        nz = int(rng.integers(48, 65))
        cells = (1000.0, 1000.0, 500.0)
        m = make_mesh(nx, ny, nz, *cells)
        f = gaussian_field((nx, ny, nz), cells, 5000.0, rng) * 100.0
        nsx = int(rng.integers(32, 129))
        nsy = int(rng.integers(32, 129))
        xs = (np.arange(nsx) + 0.5) * nx * 1000.0 / nsx
        ys = (np.arange(nsy) + 0.5) * ny * 1000.0 / nsy
        X, Y = np.meshgrid(xs, ys, indexing="xy")
        z = rng.uniform(0.0, 2000.0, X.size)
        s = np.stack([X.ravel(), Y.ravel(), z], axis=1)
        jobs.append((m, _layer_major(f)[None, :], s))
    return jobs, alphas


def moho_columns_512(seed=5):
    """Interface inversion: 512x512 columns of 0.5 km, 256x256 stations."""
    return moho_columns(seed=seed, n=512, ns_side=256, cell=500.0)


def pointmass_grid_of_mesh(mesh, rho, st):
    """A prism mesh with 2:1 horizontal:vertical cells (configs 1 and 2) on
    the reference's point-mass grid (TFM.cpp:83): node-centred cells,
    fh = 1, fv = 2 (a layer is half a grid unit), bfr = 0, densities in g/cc
    with layer 0 at the highest k, and every node a station: the stations of
    `st` at their heights over their home cells, the other nodes one grid
    unit above the top layer.  The 66.7 constant of TFM.cpp:98 assumes a
    10 km spacing, so scale = dx / 10 km.  Returns (grid, drho, surf)."""
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    kk = nz + 1 if nz % 2 == 0 else nz  # (dk-1)*fv+1 must hold every layer
    dk = (kk - 1) // 2 + 1
    g = make_grid(nx, ny, dk, 1, 2, 0, threshold=0.001, scale=mesh.dx / 10000.0)
    drho = np.zeros(nx * ny * kk)
    r = np.asarray(rho).reshape(nz, ny, nx) / 1000.0
    for l in range(nz):
        K = (kk - 1) - l - (kk - nz)
        drho[K * nx * ny:(K + 1) * nx * ny] = r[l].ravel()
    ktop = ((kk - 1) - (kk - nz)) / 2.0  # grid k of the top layer's centre
    surf = np.full(nx * ny, ktop + 0.25 + 1.0)  # the top face is half a layer above
    for x, y, z in st:
        i, j = int(x // mesh.dx), int(y // mesh.dy)
        surf[i + nx * j] = ktop + 0.25 + (z - mesh.z_top) / mesh.dx
    return g, drho, surf
