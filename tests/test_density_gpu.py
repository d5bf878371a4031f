"""GPU density builder (TFM.cpp:83-89) against its oracle restatement:
bitwise equal (same operations, no contraction), and chained into the
point-mass forward without leaving the device."""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import rel_err, tfm_density_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(61, 61, 33, 1, 2), (21, 19, 13, 1, 2), (17, 13, 9, 2, 3)])
def test_density_bitwise(ctx, dims):
    di, dj, dk, fh, fv = dims
    rc, sea, M, v = tfm_density_inputs(di, dj, dk, seed=di)
    ref = oracle.density_tfm(di, dj, dk, fh, fv, 8.0, -0.4, 0.3, rc, sea, M, v)
    out, nsel = ctx.density(di, dj, dk, sea, M, v, 8.0, -0.4, 0.3, rc, fh=fh, fv=fv)
    assert np.array_equal(out, ref)
    assert nsel == np.count_nonzero(ref)


def test_density_then_pointmass_on_device(ctx):
    torch = pytest.importorskip("torch")
    di, dj, dk = 61, 61, 33
    rc, sea, M, v = tfm_density_inputs(di, dj, dk, seed=7)
    d = lambda a: torch.tensor(a, device="cuda")
    drho, _ = ctx.density(di, dj, dk, d(sea), d(M), d(v), 8.0, -0.4, 0.3, rc)
    surf = sea + 0.3  # stations on the topography, above sea level
    g = ztm_gb300.make_grid(di, dj, dk, 1, 2, 10)
    G = ctx.pointmass(g, drho, d(surf), precision="fp64")
    ctx.sync()
    ref_d = oracle.density_tfm(di, dj, dk, 1, 2, 8.0, -0.4, 0.3, rc, sea, M, v)
    ref = oracle.pointmass_tfm(g, ref_d, surf)
    assert rel_err(G.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pointmass_model_fused(ctx, precision):
    """ztm_gfm_pointmass_model (TFM.cpp:83-99 in one call) equals the builder
    followed by the point-mass forward, and the oracle's TFM loop."""
    di, dj, dk = 61, 61, 33
    rc, sea, M, v = tfm_density_inputs(di, dj, dk, seed=11)
    surf = sea + 0.3
    g = ztm_gb300.make_grid(di, dj, dk, 1, 2, 10)
    G = ctx.pointmass_model(g, sea, M, v, surf, 8.0, -0.4, 0.3, rc, precision=precision)
    drho, _ = ctx.density(di, dj, dk, sea, M, v, 8.0, -0.4, 0.3, rc)
    G2 = ctx.pointmass(g, drho, surf, precision=precision)
    assert np.array_equal(G, G2)
    ref_d = oracle.density_tfm(di, dj, dk, 1, 2, 8.0, -0.4, 0.3, rc, sea, M, v)
    ref = oracle.pointmass_tfm(g, ref_d, surf)
    assert rel_err(G, ref) <= (1e-12 if precision == "fp64" else 1e-5)


def test_pointmass_model_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    di, dj, dk = 21, 19, 13
    rc, sea, M, v = tfm_density_inputs(di, dj, dk, seed=5)
    surf = sea + 0.2
    g = ztm_gb300.make_grid(di, dj, dk, 1, 2, 2)
    d = lambda a: torch.tensor(a, device="cuda")
    G = ctx.pointmass_model(g, d(sea), d(M), d(v), d(surf), 8.0, -0.4, 0.3, rc)
    ctx.sync()
    ref_d = oracle.density_tfm(di, dj, dk, 1, 2, 8.0, -0.4, 0.3, rc, sea, M, v)
    assert rel_err(G.cpu().numpy(), oracle.pointmass_tfm(g, ref_d, surf)) <= 1e-12
