"""Nonlinear interface inversion (L-BFGS over forward + adjoint on the GPU):
the mixed run converges like the plain double run."""
import numpy as np
import pytest

from ztm_gb300 import synth

pytestmark = pytest.mark.gpu


def test_inversion_mixed_matches_fp64_run(ctx):
    im, depth_true, rho, st, start = synth.moho_columns(seed=5, n=64, ns_side=32, cell=1000.0)
    rng = np.random.default_rng(5)
    data = ctx.interface(im, depth_true, rho, st, precision="fp64") + rng.normal(0, 0.05, len(st))
    d64, h64, n64 = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=20,
                                         precision="fp64")
    dmx, hmx, nmx = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=20,
                                         precision="mixed")
    assert n64 >= 10 and nmx >= 10
    assert h64[-1] < 0.05 * h64[0]  # the misfit falls by more than 20x
    # converged misfit of the mixed run vs the plain double run
    assert abs(hmx[-1] - h64[-1]) <= 0.02 * h64[-1] + 1e-9
    # and the mixed run's final model re-evaluated in double
    mis64 = 0.5 * np.sum((ctx.interface(im, dmx, rho, st, precision="fp64") - data) ** 2)
    assert mis64 == pytest.approx(hmx[-1], rel=1e-5)
    # the recovered interface moves towards the true one
    assert np.abs(dmx - depth_true).mean() < 0.7 * np.abs(start - depth_true).mean()
