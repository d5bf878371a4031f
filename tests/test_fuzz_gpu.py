"""Seeded random shapes through the mixed kernels: mesh sizes that are not
multiples of the tile, stage, layer-group or warp sizes, station counts that
leave partial tiles and near items, stations above, inside, beside and below
the mesh.  Each case is checked against the plain double kernels of the
library (themselves pinned to the oracle in test_prism_gpu and
test_adjoint_gpu)."""
import numpy as np
import pytest

import ztm_gb300
from helpers import rel_err

pytestmark = pytest.mark.gpu


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    nx, ny = (int(v) for v in rng.integers(1, 72, 2))
    nz = int(rng.integers(1, 41))
    dx, dy, dz = (float(v) for v in rng.uniform(200.0, 2000.0, 3))
    mesh = ztm_gb300.make_mesh(nx, ny, nz, dx, dy, dz, x0=float(rng.uniform(-5e3, 5e3)),
                               y0=float(rng.uniform(-5e3, 5e3)), z_top=float(rng.uniform(-500, 500)))
    rho = rng.normal(0.0, 250.0, nx * ny * nz)
    rho[rng.random(rho.size) < 0.2] = 0.0
    ns = int(rng.integers(1, 300))
    X1, Y1 = mesh.x0 + nx * dx, mesh.y0 + ny * dy
    Zb = mesh.z_top - nz * dz
    x = rng.uniform(mesh.x0 - 3 * dx, X1 + 3 * dx, ns)
    y = rng.uniform(mesh.y0 - 3 * dy, Y1 + 3 * dy, ns)
    kind = rng.integers(0, 4, ns)  # above, inside, below, far above
    z = np.where(kind == 0, mesh.z_top + rng.uniform(1.0, 3000.0, ns),
                 np.where(kind == 1, rng.uniform(Zb + 1.0, mesh.z_top - 1.0, ns),
                          np.where(kind == 2, Zb - rng.uniform(1.0, 2000.0, ns),
                                   mesh.z_top + rng.uniform(5e3, 5e4, ns))))
    st = np.stack([x, y, z], 1)
    return mesh, rho, st, rng


@pytest.mark.parametrize("seed", range(16))
def test_random_meshes_mixed_vs_double(ctx, seed):
    mesh, rho, st, rng = _case(seed)
    ref = ctx.prism(mesh, rho, st, precision="fp64")
    out = ctx.prism(mesh, rho, st, precision="mixed")
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= 1e-6
    r = rng.normal(0.0, 1.0, len(st))
    ga = ctx.adjoint(mesh, st, r, precision="fp64")
    gm = ctx.adjoint(mesh, st, r, precision="mixed")
    assert rel_err(gm, ga) <= 1e-6


@pytest.mark.parametrize("seed", range(4))
def test_random_batches_vs_single_calls(ctx, seed):
    jobs, refs = [], []
    for j in range(3):
        mesh, rho, st, rng = _case(100 + 3 * seed + j)
        nm = int(rng.integers(1, 20))
        models = np.stack([rho * (1.0 + 0.1 * m) for m in range(nm)])
        jobs.append((mesh, models, st))
    outs = ctx.batch(jobs)
    for (mesh, models, st), out in zip(jobs, outs):
        for m in (0, models.shape[0] - 1):
            ref = ctx.prism(mesh, models[m], st, precision="mixed")
            assert rel_err(out[m], ref) <= 1e-6


def _icase(seed):
    rng = np.random.default_rng(2000 + seed)
    nx, ny = (int(v) for v in rng.integers(1, 72, 2))
    dx, dy = (float(v) for v in rng.uniform(300.0, 3000.0, 2))
    z_base = -float(rng.uniform(20e3, 60e3))
    im = ztm_gb300.make_imesh(nx, ny, dx, dy, z_base, x0=float(rng.uniform(-5e3, 5e3)),
                              y0=float(rng.uniform(-5e3, 5e3)))
    # tops between the surface and the base; some columns thin, some shallow
    depth = rng.uniform(100.0, -z_base - 50.0, nx * ny)
    rho = rng.normal(-300.0, 80.0, nx * ny)
    ns = int(rng.integers(1, 300))
    X1, Y1 = im.x0 + nx * dx, im.y0 + ny * dy
    st = np.stack([rng.uniform(im.x0 - 2 * dx, X1 + 2 * dx, ns),
                   rng.uniform(im.y0 - 2 * dy, Y1 + 2 * dy, ns),
                   rng.uniform(-50.0, 3000.0, ns)], 1)  # some just below z = 0
    return im, depth, rho, st, rng


@pytest.mark.parametrize("seed", range(10))
def test_random_interfaces_mixed_vs_double(ctx, seed):
    """Interface columns with tops from 100 m below the surface to the base:
    stations near shallow tops take the double near path."""
    im, depth, rho, st, rng = _icase(seed)
    ref = ctx.interface(im, depth, rho, st, precision="fp64")
    out = ctx.interface(im, depth, rho, st, precision="mixed")
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= 1e-6
    r = rng.normal(0.0, 1.0, len(st))
    gr64, gd64 = ctx.interface_adjoint(im, depth, rho, st, r, precision="fp64")
    grm, gdm = ctx.interface_adjoint(im, depth, rho, st, r, precision="mixed")
    assert rel_err(grm, gr64) <= 1e-5 and rel_err(gdm, gd64) <= 1e-5


@pytest.mark.parametrize("seed", range(3))
def test_station_order_does_not_change_the_fields(ctx, seed):
    """The forwards compute the stations in Z order of their home cells, so a
    permuted station list gives the permuted field.  Only stations that share
    a home cell can land in other warps, where a warp vote may pick the other
    far-field form: the tolerance is the second-order form's truncation."""
    mesh, rho, st, rng = _case(200 + seed)
    perm = rng.permutation(len(st))
    out = ctx.prism(mesh, rho, st, precision="mixed")
    outp = ctx.prism(mesh, rho, st[perm], precision="mixed")
    assert rel_err(outp, out[perm]) <= 1e-8
    im, depth, rc, ist, rng = _icase(200 + seed)
    perm = rng.permutation(len(ist))
    out = ctx.interface(im, depth, rc, ist, precision="mixed")
    outp = ctx.interface(im, depth, rc, ist[perm], precision="mixed")
    assert rel_err(outp, out[perm]) <= 1e-8


def test_stations_sharing_one_home_cell(ctx):
    """Every station in one cell column (equal sort keys, one near box for
    all), above and inside the mesh: the mixed forward and adjoint against
    the double kernels."""
    rng = np.random.default_rng(77)
    mesh = ztm_gb300.make_mesh(40, 36, 20, 800.0, 900.0, 400.0)
    rho = rng.normal(0.0, 250.0, 40 * 36 * 20)
    ns = 500
    x = mesh.x0 + 17 * 800.0 + rng.uniform(1.0, 799.0, ns)
    y = mesh.y0 + 11 * 900.0 + rng.uniform(1.0, 899.0, ns)
    z = np.where(rng.random(ns) < 0.5, mesh.z_top + rng.uniform(1.0, 2000.0, ns),
                 mesh.z_top - rng.uniform(1.0, 7999.0, ns))
    st = np.stack([x, y, z], 1)
    ref = ctx.prism(mesh, rho, st, precision="fp64")
    assert rel_err(ctx.prism(mesh, rho, st, precision="mixed"), ref) <= 1e-6
    r = rng.normal(0.0, 1.0, ns)
    assert rel_err(ctx.adjoint(mesh, st, r, precision="mixed"),
                   ctx.adjoint(mesh, st, r, precision="fp64")) <= 1e-6


def test_many_stations_on_a_small_mesh(ctx):
    """200,003 stations (1,563 station tiles, 6,251 near items, many equal
    sort keys) over a 16x12x8 mesh: mixed against the double kernel."""
    rng = np.random.default_rng(88)
    mesh = ztm_gb300.make_mesh(16, 12, 8, 700.0, 600.0, 350.0, x0=-2000.0, y0=1000.0)
    rho = rng.normal(0.0, 250.0, 16 * 12 * 8)
    ns = 200_003
    st = np.stack([rng.uniform(-4000.0, 11000.0, ns), rng.uniform(0.0, 9000.0, ns),
                   rng.uniform(-2500.0, 1500.0, ns)], 1)
    ref = ctx.prism(mesh, rho, st, precision="fp64")
    out = ctx.prism(mesh, rho, st, precision="mixed")
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= 1e-6
