"""Failure handling on the GPU without a GPU fault.

Every copy-arrival wait of the mixed forward's far kernel is bounded; a wait
that gives up makes its block record a timeout in the context's error word,
wait (with the full bound) for the copies it still has in flight, and stop.
The test hook ztm_ctx_test_timeout points each stage wait at a barrier that
nothing completes, with a bound of a few tests, so that the waits run out:
the call must return ZTM_ERR_TIMEOUT, and the next call on the same context,
without the hook, must run normally.  Nothing here faults, traps or hangs
the GPU: the density copies land as usual and each block waits for its own
before it stops."""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import awkward_stations, rel_err, small_mesh

pytestmark = pytest.mark.gpu


def test_timeout_is_reported_and_the_context_recovers(ctx):
    mesh, rho = small_mesh(96, 80, 24, seed=4)
    st = awkward_stations(mesh, n_random=300)
    ref = oracle.prism_mesh(mesh, rho, st)
    ctx.test_timeout(4)
    try:
        with pytest.raises(ztm_gb300.GravityError) as e:
            ctx.prism(mesh, rho, st, precision="mixed")
        assert e.value.code == ztm_gb300.ERR_TIMEOUT
    finally:
        ctx.test_timeout(0)
    out = ctx.prism(mesh, rho, st, precision="mixed")
    assert rel_err(out, ref) <= 1e-6
    # the error word was cleared: a device-pointer call reports nothing stale
    torch = pytest.importorskip("torch")
    out = ctx.prism(mesh, torch.tensor(rho, device="cuda"), torch.tensor(st, device="cuda"),
                    precision="mixed")
    ctx.sync()
    assert rel_err(out.cpu().numpy(), ref) <= 1e-6


def test_batched_tensor_core_timeout_frees_the_block_and_recovers(ctx):
    """The tensor-core far items of the batched launch under the same hook:
    the stage waits run out, each block waits for its copies and MMAs in
    flight, frees its tensor memory and stops; the call reports the timeout
    and the next batched call (hook off, a new graph) gives the field of
    single calls, so no tensor memory was left allocated."""
    rng = np.random.default_rng(3)
    mesh, rho = small_mesh(64, 56, 16, seed=6)
    models = np.stack([rho * (1.0 + 0.05 * k) + rng.normal(0, 2, rho.size) for k in range(8)])
    st = awkward_stations(mesh, n_random=400)
    ctx.test_timeout(4)
    try:
        with pytest.raises(ztm_gb300.GravityError) as e:
            ctx.batch([(mesh, models, st)])
        assert e.value.code == ztm_gb300.ERR_TIMEOUT
    finally:
        ctx.test_timeout(0)
    out = ctx.batch([(mesh, models, st)])[0]
    for k in (0, 7):
        ref = ctx.prism(mesh, models[k], st, precision="mixed")
        assert rel_err(out[k], ref) <= 1e-6
