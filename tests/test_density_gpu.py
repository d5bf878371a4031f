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
