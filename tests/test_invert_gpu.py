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


def test_gauss_newton_converges_further_than_lbfgs(ctx):
    """Gauss-Newton with CG inner solves (J v and J^T w products): in 10
    outer iterations it gets the misfit well below what 20 L-BFGS iterations
    reach, in mixed precision as in double, and the two runs agree."""
    im, depth_true, rho, st, start = synth.moho_columns(seed=5, n=64, ns_side=32, cell=1000.0)
    rng = np.random.default_rng(5)
    data = ctx.interface(im, depth_true, rho, st, precision="fp64") + rng.normal(0, 0.05, len(st))
    _, hl, _ = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=20,
                                    precision="mixed")
    dg, hg, ng = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=10,
                                      precision="mixed", method="gn", cg_iterations=10)
    d64, h64, n64 = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=10,
                                         precision="fp64", method="gn", cg_iterations=10)
    assert ng >= 5 and n64 >= 5
    assert hg[-1] < 0.5 * hl[-1]
    assert abs(hg[-1] - h64[-1]) <= 0.02 * h64[-1] + 1e-9
    assert np.abs(dg - depth_true).mean() < 0.5 * np.abs(start - depth_true).mean()
