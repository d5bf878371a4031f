"""The damped Gauss-Newton step of the reference's optimiser on the GPU
(ztm_lm_steps) against the reference's own code: zmath.cpp compiled
unchanged (MTM, inv, T and its operators) with the two statements of
LMA::fit (TFM.cpp:159-160), or their numpy restatement where the reference
sources are absent.

TOLERANCES: J^T J 1e-13 (normwise relative: the same sums in another order);
the trial models 1e-9 (normwise relative over b's change: the reference
inverts and multiplies, the library factorises with the right-hand side
attached, and the normal equations square the condition number)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def reference(J, r, b, sig, dm):
    if oracle.ref_lm_available():
        return oracle.ref_lm_steps(J, r, b, sig, dm)
    return oracle.lm_steps(J, r, b, sig, dm)


def problem(nrows, ncols, seed):
    rng = np.random.default_rng(seed)
    J = rng.normal(size=(nrows, ncols)) * rng.uniform(0.1, 10.0, ncols)[None, :]
    r = rng.normal(size=nrows)
    b = rng.normal(size=ncols)
    sig = rng.uniform(0.05, 2.0, ncols)
    dm = np.array([[0.0, 0.0], [1e-3, 1e-4], [0.1, 1e-2], [1.0, 1.0]])
    return J, r, b, sig, dm


@pytest.mark.parametrize("nrows,ncols", [(400, 60), (2000, 300), (150, 130)])
def test_lm_steps_match_reference(ctx, nrows, ncols):
    J, r, b, sig, dm = problem(nrows, ncols, nrows + ncols)
    Bref, JJref = reference(J, r, b, sig, dm)
    B, JJ = ctx.lm_steps(J, r, b, sig, dm, return_jtj=True)
    assert np.max(np.abs(JJ - JJref)) <= 1e-13 * np.max(np.abs(JJref))
    for d in range(dm.shape[0]):
        step_ref = Bref[d] - b
        assert np.max(np.abs((B[d] - b) - step_ref)) <= 1e-9 * np.max(np.abs(step_ref)), d


def test_lm_singular_system_keeps_b(ctx):
    """A parameter the data do not constrain (zero column) and no damping:
    the reference's inv returns zeros, so the trial is b itself."""
    J, r, b, sig, _ = problem(300, 40, 7)
    J[:, 5] = 0.0
    dm = np.array([[0.0, 0.0], [0.0, 1e-2]])
    Bref, _ = reference(J, r, b, sig, dm)
    B = ctx.lm_steps(J, r, b, sig, dm)
    assert np.array_equal(B[0], b) and np.array_equal(Bref[0], b)
    step_ref = Bref[1] - b
    assert np.max(np.abs((B[1] - b) - step_ref)) <= 1e-9 * np.max(np.abs(step_ref))


def test_lm_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    J, r, b, sig, dm = problem(500, 70, 3)
    host = ctx.lm_steps(J, r, b, sig, dm)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    dev = ctx.lm_steps(d(J), d(r), d(b), d(sig), d(dm))
    ctx.sync()
    assert np.array_equal(dev.cpu().numpy(), host)


def test_lm_underdetermined_and_one_parameter(ctx):
    """Fewer data than parameters: J^T J has rank 20 of 50, and the damping
    of the uncertainties (d1 > 0) makes the system solvable; and the smallest
    system, one parameter."""
    J, r, b, sig, _ = problem(20, 50, 9)
    dm = np.array([[0.0, 0.5], [0.3, 0.5]])
    Bref, _ = reference(J, r, b, sig, dm)
    B = ctx.lm_steps(J, r, b, sig, dm)
    for d in (0, 1):
        step_ref = Bref[d] - b
        assert np.max(np.abs((B[d] - b) - step_ref)) <= 1e-8 * np.max(np.abs(step_ref)), d
    J1 = np.arange(1.0, 8.0).reshape(7, 1)
    r1 = np.linspace(-1.0, 1.0, 7) + 0.3
    B1 = ctx.lm_steps(J1, r1, np.array([2.0]), np.array([0.5]), np.array([[0.1, 0.2]]))
    jj, jr = float(np.sum(J1 ** 2)), float(np.dot(J1[:, 0], r1))
    want = 2.0 + jr / (jj + 0.1 * jj + 0.2 / 0.25)
    assert B1[0, 0] == pytest.approx(want, rel=1e-14)


def test_lm_steps_beyond_the_shared_memory_panel(ctx):
    """3,520 parameters: more rows than a panel in shared memory holds, so
    the panels are factorised in global memory (row swaps over whole rows);
    each step against numpy's solve of the same damped system built from the
    library's own J^T J."""
    rng = np.random.default_rng(77)
    nrows, ncols = 3600, 3520
    J = rng.normal(size=(nrows, ncols)) * rng.uniform(0.5, 2.0, ncols)[None, :]
    r, b = rng.normal(size=nrows), rng.normal(size=ncols)
    sig = rng.uniform(0.5, 2.0, ncols)
    dm = np.array([[1e-3, 1e-3], [0.1, 1.0]])
    B, JJ = ctx.lm_steps(J, r, b, sig, dm, return_jtj=True)
    g = J.T @ r
    for k, (d0, d1) in enumerate(dm):
        A = JJ + np.diag(d0 * np.diag(JJ) + d1 / sig ** 2)
        step = np.linalg.solve(A, g)
        assert np.max(np.abs((B[k] - b) - step)) <= 1e-9 * np.max(np.abs(step)), k
