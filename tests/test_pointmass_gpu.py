"""Point-mass model (the reference's algorithm) on the GPU against the
reference's own CPU lambda (TFM.cpp:95-99 compiled from TFM.cpp), the oracle
restatement of it, and the reference GF kernel."""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import rel_err, tfm_like_inputs
from ztm_gb300 import synth

pytestmark = pytest.mark.gpu

# TOLERANCES: double path vs TFM.cpp restatement 1e-12 (normwise relative);
# float path vs double 1e-5 (float rounding and summation order).
TOL64 = 1e-12
TOL32 = 1e-5


@pytest.mark.parametrize("dims", [(31, 29, 17, 1, 2, 5), (61, 61, 33, 1, 2, 10), (9, 7, 5, 2, 3, 1),
                                  (5, 5, 2, 1, 1, 0)])
def test_fp64_matches_tfm_restatement(ctx, dims):
    di, dj, dk, fh, fv, bfr = dims
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
    drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=di)
    ref = oracle.pointmass_tfm(g, drho, surf)
    out = ctx.pointmass(g, drho, surf, precision="fp64")
    assert rel_err(out, ref) <= TOL64
    interior = np.zeros((dj, di), bool)
    interior[bfr:dj - bfr, bfr:di - bfr] = True
    assert np.all(out.reshape(dj, di)[~interior] == 0.0)


def test_fp32_matches_tfm_restatement(ctx):
    g = ztm_gb300.make_grid(31, 29, 17, 1, 2, 5)
    drho, surf = tfm_like_inputs(31, 29, 17, seed=3)
    ref = oracle.pointmass_tfm(g, drho, surf)
    out = ctx.pointmass(g, drho, surf, precision="fp32")
    assert rel_err(out, ref) <= TOL32


def test_explicit_node_list(ctx):
    g = ztm_gb300.make_grid(21, 19, 9, 1, 2, 3)
    drho, surf = tfm_like_inputs(21, 19, 9, seed=4)
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    ref = oracle.pointmass_tfm(g, drho, surf, nn=nn)
    out = ctx.pointmass(g, drho, surf, nn=nn, precision="fp64")
    assert rel_err(out, ref) <= TOL64


def test_scale_and_empty(ctx):
    g = ztm_gb300.make_grid(11, 11, 5, 1, 2, 2, scale=0.2)
    drho, surf = tfm_like_inputs(11, 11, 5, seed=5)
    out = ctx.pointmass(g, np.zeros_like(drho), surf)
    assert np.all(out == 0)
    ref = oracle.pointmass_tfm(g, drho, surf)
    assert rel_err(ctx.pointmass(g, drho, surf), ref) <= TOL64


def test_all_stations_in_buffer(ctx):
    g = ztm_gb300.make_grid(8, 8, 4, 1, 2, 4)  # bfr leaves no interior
    drho, surf = tfm_like_inputs(8, 8, 4, seed=6)
    out = ctx.pointmass(g, drho, surf)
    assert out.shape == (64,) and np.all(out == 0)


def test_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    g = ztm_gb300.make_grid(31, 29, 17, 1, 2, 5)
    drho, surf = tfm_like_inputs(31, 29, 17, seed=7)
    ref = oracle.pointmass_tfm(g, drho, surf)
    out = ctx.pointmass(g, torch.tensor(drho, device="cuda"), torch.tensor(surf, device="cuda"))
    ctx.sync()
    assert rel_err(out.cpu().numpy(), ref) <= TOL64


@pytest.mark.skipif(not oracle.ref_gf_available(), reason="reference GF image not built here")
def test_reference_gf_kernel_agrees(ctx):
    """The unchanged reference kernel, float with atomics, vs the oracle."""
    g = ztm_gb300.make_grid(61, 61, 33, 1, 2, 10)
    drho, surf = tfm_like_inputs(61, 61, 33, seed=8)
    ref = oracle.pointmass_tfm(g, drho, surf)
    gf, _ = oracle.ref_gf(g, drho.astype(np.float32), surf.astype(np.float32))
    # the reference accumulates in float in atomic order: ~1e-5 normwise
    assert rel_err(gf, ref) <= 5e-5
    ours = ctx.pointmass(g, drho, surf, precision="fp32")
    assert rel_err(ours, ref) <= TOL32


@pytest.mark.parametrize("dims", [(31, 29, 17, 1, 2, 5), (9, 7, 5, 2, 3, 1), (5, 5, 2, 1, 1, 0),
                                  (40, 3, 9, 1, 2, 1)])
def test_fp32_dims_and_node_lists(ctx, dims):
    """The float path by node columns: grids with fh, fv > 1, thin grids, and
    explicit node lists (a node listed twice counts twice, as in the loop of
    TFM.cpp:96-98)."""
    di, dj, dk, fh, fv, bfr = dims
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
    drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=di + 1)
    ref = oracle.pointmass_tfm(g, drho, surf)
    assert rel_err(ctx.pointmass(g, drho, surf, precision="fp32"), ref) <= TOL32
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    nn2 = np.concatenate([nn, nn[::3]])
    ref2 = oracle.pointmass_tfm(g, drho, surf, nn=nn2)
    assert rel_err(ctx.pointmass(g, drho, surf, nn=nn2, precision="fp32"), ref2) <= TOL32


def test_bad_node_index_on_device_is_reported(ctx):
    """A node index outside the grid passed in device memory is skipped on
    the device and reported as a range error at the call's end."""
    torch = pytest.importorskip("torch")
    g = ztm_gb300.make_grid(21, 19, 9, 1, 2, 3)
    drho, surf = tfm_like_inputs(21, 19, 9, seed=9)
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    nn[len(nn) // 2] = drho.size + 7
    with pytest.raises(ztm_gb300.GravityError):
        ctx.pointmass(g, torch.tensor(drho, device="cuda"), torch.tensor(surf, device="cuda"),
                      nn=torch.tensor(nn, device="cuda"), precision="fp32")
        ctx.sync()


needs_ref_tfm = pytest.mark.skipif(not oracle.ref_tfm_available(),
                                   reason="reference TFM.cpp lambda not built")


@needs_ref_tfm
@pytest.mark.parametrize("dims", [(16, 16, 9, 1, 3, 0), (31, 29, 17, 1, 2, 5),
                                  (61, 61, 33, 1, 2, 10), (21, 19, 9, 2, 2, 3)])
def test_fp64_matches_reference_lambda(ctx, dims):
    """The double path against the reference's own compiled lambda (the
    golden dims of tests/golden and TFM's 61x61x33), with its threshold list
    and with an explicit list holding duplicates."""
    di, dj, dk, fh, fv, bfr = dims
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
    drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=3 * di + dk)
    ref = oracle.ref_tfm(g, drho, surf)
    assert rel_err(ctx.pointmass(g, drho, surf, precision="fp64"), ref) <= TOL64
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    nn = np.concatenate([nn, nn[::4]])
    ref = oracle.ref_tfm(g, drho, surf, nn=nn)
    assert rel_err(ctx.pointmass(g, drho, surf, nn=nn, precision="fp64"), ref) <= TOL64


@needs_ref_tfm
def test_fp64_plain_mesh_on_reference_grid(ctx):
    """The 64x64x32 plain mesh (2x2x1 km cells) on the reference's node grid
    (h = 2 km, fv = 2, every node a station): the double path against the
    compiled reference lambda, normwise and per station (stations whose
    field is not near a zero crossing)."""
    mesh, rho, st = synth.plain_mesh_64x64x32()
    g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
    ref = oracle.ref_tfm(g, drho, surf)
    out = ctx.pointmass(g, drho, surf, precision="fp64")
    assert rel_err(out, ref) <= TOL64
    big = np.abs(ref) > 1e-3 * np.abs(ref).max()
    assert np.max(np.abs(out - ref)[big] / np.abs(ref)[big]) <= 1e-10
