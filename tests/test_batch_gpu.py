"""Batched persistent launch vs one-at-a-time calls (same mixed method)."""
import numpy as np
import pytest

import ztm_gb300
from helpers import rel_err, small_mesh

pytestmark = pytest.mark.gpu


def test_batch_matches_single_calls(ctx):
    rng = np.random.default_rng(0)
    jobs = []
    for shape in [(40, 32, 12), (17, 23, 5), (64, 48, 10)]:
        mesh, rho = small_mesh(*shape, seed=sum(shape))
        nm = 1 + shape[2] % 11
        models = np.stack([rho * (1 + 0.1 * k) + rng.normal(0, 5, rho.size) for k in range(nm)])
        ns = 50 + shape[0]
        st = np.stack([rng.uniform(mesh.x0, mesh.x0 + mesh.nx * mesh.dx, ns),
                       rng.uniform(mesh.y0, mesh.y0 + mesh.ny * mesh.dy, ns),
                       rng.uniform(mesh.z_top, mesh.z_top + 2000, ns)], 1)
        jobs.append((mesh, models, st))
    outs = ctx.batch(jobs)
    for (mesh, models, st), out in zip(jobs, outs):
        for k in range(models.shape[0]):
            ref = ctx.prism(mesh, models[k], st, precision="mixed")
            assert rel_err(out[k], ref) <= 1e-6
    # replay of the cached graph gives bitwise the same result
    outs2 = ctx.batch(jobs)
    for a, b in zip(outs, outs2):
        assert np.array_equal(a, b)


def test_batch_line_search_trials(ctx):
    mesh, rho = small_mesh(48, 40, 16, seed=5)
    _, p = small_mesh(48, 40, 16, seed=6)
    alphas = np.linspace(0, 2, 32)
    trials = rho[None, :] + alphas[:, None] * p[None, :]
    st = np.stack(np.meshgrid(np.arange(20) * 2000.0 + 500, np.arange(16) * 2000.0 + 1700), -1).reshape(-1, 2)
    st = np.concatenate([st, np.full((len(st), 1), 300.0)], 1)
    out = ctx.batch([(mesh, trials, st)])[0]
    g0 = ctx.prism(mesh, rho, st, precision="fp64")
    gp = ctx.prism(mesh, p, st, precision="fp64")
    for k, a in enumerate(alphas):
        assert rel_err(out[k], g0 + a * gp) <= 1e-6


def test_batch_autotuned_shape_gives_the_same_field(ctx):
    """With the autotuner the shape is measured on the first call and cached;
    every shape computes the same sums (grouping of float partials aside)."""
    rng = np.random.default_rng(2)
    mesh, rho = small_mesh(40, 36, 16, seed=9)
    models = np.stack([rho * (1 + 0.05 * k) for k in range(10)])
    st = np.stack([rng.uniform(mesh.x0, mesh.x0 + 40e3, 90),
                   rng.uniform(mesh.y0, mesh.y0 + 28.8e3, 90),
                   rng.uniform(mesh.z_top + 10.0, mesh.z_top + 2500.0, 90)], 1)
    ref = ctx.batch([(mesh, models, st)])[0]
    tuned = ctx.batch([(mesh, models, st)], autotune=True)[0]
    again = ctx.batch([(mesh, models, st)], autotune=True)[0]
    assert rel_err(tuned, ref) <= 1e-6
    assert np.array_equal(tuned, again)


def test_batch_awkward_stations_with_padded_layers(ctx):
    """Multi-model far items (tensor cores) with 13 layers (padded to 16) and
    stations on faces, edges and vertices, inside the mesh and below it (one
    at the centre of the first padding layer under a column, where the
    padded layer's far-field value would be 0/0 without the mask): every
    model against its single mixed call."""
    from helpers import awkward_stations
    rng = np.random.default_rng(11)
    mesh, rho = small_mesh(20, 18, 13, seed=12)
    models = np.stack([rho * (1.0 + 0.07 * k) + rng.normal(0, 3, rho.size) for k in range(5)])
    st = awkward_stations(mesh, n_random=150, seed=13)
    out = ctx.batch([(mesh, models, st)])[0]
    assert np.all(np.isfinite(out))
    for k in range(models.shape[0]):
        ref = ctx.prism(mesh, models[k], st, precision="mixed")
        assert rel_err(out[k], ref) <= 1e-6, k


def test_batch_more_models_than_a_tensor_core_group(ctx):
    """37 models: two 32-model groups of tensor-core far items, the second
    with 5 models and 27 zero-padded ones; every model against its single
    mixed call, and a 2-model job beside it in the same launch."""
    rng = np.random.default_rng(21)
    mesh, rho = small_mesh(36, 30, 16, seed=22)
    models = np.stack([rho * (1.0 + 0.03 * k) + rng.normal(0, 4, rho.size) for k in range(37)])
    st = np.stack([rng.uniform(mesh.x0 - 3e3, mesh.x0 + 39e3, 140),
                   rng.uniform(mesh.y0 - 3e3, mesh.y0 + 27e3, 140),
                   rng.uniform(mesh.z_top + 5.0, mesh.z_top + 2500.0, 140)], 1)
    mesh2, rho2 = small_mesh(24, 20, 12, seed=23)
    two = np.stack([rho2, -0.5 * rho2])
    outs = ctx.batch([(mesh, models, st), (mesh2, two, st)])
    for k in (0, 17, 31, 32, 36):
        ref = ctx.prism(mesh, models[k], st, precision="mixed")
        assert rel_err(outs[0][k], ref) <= 1e-6, k
    ref2 = ctx.prism(mesh2, rho2, st, precision="mixed")
    assert rel_err(outs[1][0], ref2) <= 1e-6
    assert rel_err(outs[1][1], -0.5 * ref2) <= 1e-6


def test_batch_deep_mesh_runs_on_the_cuda_cores(ctx):
    """300 layers: the tensor-core items' column stages (768 bytes a layer)
    would not fit in shared memory, so the launch takes the CUDA-core
    variant; every model against its single mixed call."""
    rng = np.random.default_rng(31)
    mesh, rho = small_mesh(10, 8, 300, seed=32)
    models = np.stack([rho, 0.5 * rho + rng.normal(0, 3, rho.size), -rho])
    st = np.stack([rng.uniform(mesh.x0, mesh.x0 + 10e3, 40), rng.uniform(mesh.y0, mesh.y0 + 6.4e3, 40),
                   rng.uniform(mesh.z_top + 5.0, mesh.z_top + 1500.0, 40)], 1)
    out = ctx.batch([(mesh, models, st)])[0]
    for k in range(3):
        ref = ctx.prism(mesh, models[k], st, precision="mixed")
        assert rel_err(out[k], ref) <= 1e-6, k
