"""Prism forward on the GPU against the double-precision oracle.

TOLERANCES (normwise relative, max|a-ref|/max|ref|):
  plain FP64 kernel vs oracle      1e-10  (same closed form; the far-field
                                           cancellation of the 8-corner sum
                                           amplifies last-bit differences of
                                           log/atan between libm and CUDA)
  mixed kernel vs FP64             1e-6   (the precision target)
  float kernel vs FP64             1e-3
"""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import awkward_stations, rel_err, small_mesh

pytestmark = pytest.mark.gpu
TOL64 = 1e-10
TOLMIX = 1e-6
TOL32 = 1e-3


@pytest.mark.parametrize("shape", [(12, 10, 6), (1, 1, 1), (7, 3, 11), (33, 17, 5)])
def test_fp64_matches_oracle(ctx, shape):
    mesh, rho = small_mesh(*shape, seed=sum(shape))
    st = awkward_stations(mesh)
    ref = oracle.prism_mesh(mesh, rho, st)
    out = ctx.prism(mesh, rho, st, precision="fp64")
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= TOL64


@pytest.mark.parametrize("shape", [(12, 10, 6), (40, 36, 16), (64, 48, 10)])
def test_mixed_matches_oracle(ctx, shape):
    mesh, rho = small_mesh(*shape, seed=3)
    st = awkward_stations(mesh, n_random=60)
    ref = oracle.prism_mesh(mesh, rho, st)
    out = ctx.prism(mesh, rho, st, precision="mixed")
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= TOLMIX


def test_fp32_mode(ctx):
    mesh, rho = small_mesh(40, 36, 16, seed=4)
    st = awkward_stations(mesh)
    ref = oracle.prism_mesh(mesh, rho, st)
    assert rel_err(ctx.prism(mesh, rho, st, precision="fp32"), ref) <= TOL32


@pytest.mark.parametrize("q", [3.0, 4.0, 6.0, 10.0])
def test_mixed_near_threshold_option(ctx, q):
    mesh, rho = small_mesh(48, 40, 12, seed=5)
    st = awkward_stations(mesh, n_random=30)
    ref = ctx.prism(mesh, rho, st, precision="fp64")
    tol = TOLMIX if q >= 4 else 1e-4
    assert rel_err(ctx.prism(mesh, rho, st, precision="mixed", near_q=q), ref) <= tol


def test_list_matches_mesh(ctx):
    mesh, rho = small_mesh(9, 8, 5, seed=6)
    st = awkward_stations(mesh, n_random=20)
    geom = []
    for l in range(mesh.nz):
        for iy in range(mesh.ny):
            for ix in range(mesh.nx):
                geom.append((mesh.x0 + ix * mesh.dx, mesh.x0 + (ix + 1) * mesh.dx,
                             mesh.y0 + iy * mesh.dy, mesh.y0 + (iy + 1) * mesh.dy,
                             mesh.z_top - (l + 1) * mesh.dz, mesh.z_top - l * mesh.dz))
    geom = np.array(geom)
    ref = oracle.prism_list(geom, rho, st)
    assert rel_err(ctx.prism_list(geom, rho, st, precision="fp64"), ref) <= TOL64
    assert rel_err(ctx.prism_list(geom, rho, st, precision="mixed"), ref) <= TOLMIX
    assert rel_err(ref, oracle.prism_mesh(mesh, rho, st)) <= 1e-13


def test_list_irregular_prisms(ctx):
    rng = np.random.default_rng(7)
    n = 500
    x0 = rng.uniform(-50e3, 50e3, n)
    y0 = rng.uniform(-50e3, 50e3, n)
    z1 = rng.uniform(-20e3, 0.0, n)
    geom = np.stack([x0, x0 + rng.uniform(100, 5000, n), y0, y0 + rng.uniform(100, 5000, n),
                     z1 - rng.uniform(100, 3000, n), z1], axis=1)
    rho = rng.normal(0, 300, n)
    st = np.stack([rng.uniform(-60e3, 60e3, 50), rng.uniform(-60e3, 60e3, 50),
                   rng.uniform(0, 2000, 50)], axis=1)
    ref = oracle.prism_list(geom, rho, st)
    assert rel_err(ctx.prism_list(geom, rho, st, precision="fp64"), ref) <= TOL64
    assert rel_err(ctx.prism_list(geom, rho, st, precision="mixed"), ref) <= TOLMIX


def test_zero_density_and_single_station(ctx):
    mesh, rho = small_mesh(10, 10, 4)
    st = np.array([[100.0, 2000.0, 500.0]])
    assert np.all(ctx.prism(mesh, np.zeros_like(rho), st, precision="mixed") == 0)
    ref = oracle.prism_mesh(mesh, rho, st)
    for p in ("fp64", "mixed"):
        assert rel_err(ctx.prism(mesh, rho, st, precision=p), ref) <= TOLMIX


def test_linearity_in_density(ctx):
    mesh, rho = small_mesh(64, 48, 10, seed=8)
    _, rho2 = small_mesh(64, 48, 10, seed=9)
    st = awkward_stations(mesh)
    a = ctx.prism(mesh, rho, st, precision="mixed")
    b = ctx.prism(mesh, rho2, st, precision="mixed")
    c = ctx.prism(mesh, 2.0 * rho - 0.5 * rho2, st, precision="mixed")
    assert rel_err(c, 2.0 * a - 0.5 * b) <= 1e-7


def test_draped_mesh_256_mixed_vs_fp64_subset(ctx):
    """The full 256x256x64 draped mesh; the double kernel on a station subset."""
    from ztm_gb300 import synth
    mesh, rho, st = synth.draped_mesh_256x256x64()
    sub = st[np.random.default_rng(0).choice(len(st), 48, replace=False)]
    ref = ctx.prism(mesh, rho, sub, precision="fp64")
    out = ctx.prism(mesh, rho, sub, precision="mixed")
    assert rel_err(out, ref) <= TOLMIX
    full = ctx.prism(mesh, rho, st, precision="mixed")
    assert np.all(np.isfinite(full))
    idx = {tuple(r): i for i, r in enumerate(st)}
    pick = [idx[tuple(r)] for r in sub]
    assert rel_err(full[pick], out) <= 1e-7  # chunking differs with the station count


def test_autotuned_shape_gives_the_same_field(ctx):
    mesh, rho = small_mesh(96, 80, 16, seed=11)
    st = awkward_stations(mesh, n_random=300)
    ref = ctx.prism(mesh, rho, st, precision="mixed")
    a = ctx.prism(mesh, rho, st, precision="mixed", autotune=True)  # tunes and caches
    b = ctx.prism(mesh, rho, st, precision="mixed", autotune=True)  # cached shape
    assert np.array_equal(a, b)
    assert rel_err(a, ref) <= 1e-7  # only the summation grouping differs


def test_plain_mesh_64_full_size_vs_oracle(ctx):
    """64x64x32 prisms of 2x2x1 km, 32x32 stations at +100 m:
    the plain double kernel and the mixed kernel against the CPU oracle on
    every station."""
    from ztm_gb300 import synth
    mesh, rho, st = synth.plain_mesh_64x64x32()
    ref = oracle.prism_mesh(mesh, rho, st)
    assert rel_err(ctx.prism(mesh, rho, st, precision="fp64"), ref) <= TOL64
    assert rel_err(ctx.prism(mesh, rho, st, precision="mixed"), ref) <= TOLMIX


def test_draped_mesh_256_linearity_and_batch(ctx):
    """Size-independent checks on the full 256x256x64 draped mesh (every
    station): the mixed forward is linear in the density, and a trial model
    of a batched launch equals the single call."""
    from ztm_gb300 import synth
    mesh, rho, st = synth.draped_mesh_256x256x64()
    rho2 = np.random.default_rng(12).normal(0.0, 150.0, rho.size)
    a = ctx.prism(mesh, rho, st, precision="mixed")
    b = ctx.prism(mesh, rho2, st, precision="mixed")
    c = ctx.prism(mesh, 2.0 * rho - 0.5 * rho2, st, precision="mixed")
    assert rel_err(c, 2.0 * a - 0.5 * b) <= 1e-7
    trials = np.stack([rho + al * rho2 for al in (0.0, 0.5, 1.0)])
    out = ctx.batch([(mesh, trials, st)])[0]
    ref = ctx.prism(mesh, trials[1], st, precision="mixed")
    assert rel_err(out[1], ref) <= 1e-6
    assert rel_err(out[0], a) <= 1e-6


@pytest.mark.parametrize("shape", [(40, 36, 16), (96, 80, 20)])
def test_form_counts_cover_every_slot(ctx, shape):
    """The counting variant of the far kernel (the numerators of the
    executed-flop roofline) gives the same field to the bit, and its slots
    add up to every station x column x padded layer; the near regions'
    corner evaluations are counted where stations sit on the mesh."""
    mesh, rho = small_mesh(*shape, seed=5)
    st = awkward_stations(mesh, n_random=200)
    gz = ctx.prism(mesh, rho, st, precision="mixed")
    ctx.count_forms(True)
    try:
        gz_c = ctx.prism(mesh, rho, st, precision="mixed")
        counts = ctx.form_counts()
    finally:
        ctx.count_forms(False)
    assert np.array_equal(gz, gz_c)
    nzp = (mesh.nz + 7) // 8 * 8
    assert counts[0] + counts[1] + counts[2] == len(st) * mesh.nx * mesh.ny * nzp
    assert counts[3] > 0
    assert ctx.form_counts() == (0, 0, 0, 0)  # read clears


def test_column_pairs_over_padding_layers(ctx):
    """nz = 13 (three zero-density padding layers in each 16-layer column):
    warps whose stations all lie above the mesh bottom take two far columns
    per pass over all padded layers, a warp with a station below the bottom
    keeps the masked single-column path; the field matches the oracle and
    the counters show column pairs."""
    mesh, rho = small_mesh(120, 24, 13, seed=9)
    rng = np.random.default_rng(9)
    n = 95
    st = np.stack([rng.uniform(mesh.x0, mesh.x0 + 10 * mesh.dx, n),
                   rng.uniform(mesh.y0, mesh.y0 + mesh.ny * mesh.dy, n),
                   rng.uniform(mesh.z_top + 10.0, mesh.z_top + 2000.0, n)], axis=1)
    below = [mesh.x0 + 4.5 * mesh.dx, mesh.y0 + 10.5 * mesh.dy,
             mesh.z_top - mesh.nz * mesh.dz - 0.5 * mesh.dz]
    st = np.vstack([st, below])
    ref = oracle.prism_mesh(mesh, rho, st)
    ctx.count_forms(True)
    try:
        out = ctx.prism(mesh, rho, st, precision="mixed")
        counts = ctx.form_counts()
    finally:
        ctx.count_forms(False)
    assert np.all(np.isfinite(out))
    assert rel_err(out, ref) <= TOLMIX
    assert counts[2] > 0
    assert counts[0] + counts[1] + counts[2] == len(st) * mesh.nx * mesh.ny * 16
