"""The workloads at their full sizes, checked against double precision on
every station (or on every regional mesh), not on subsets.

  256x256x64 draped mesh, 128x128 stations: the mixed field and the plain
    double field at all 16,384 stations against the committed field of the
    CPU oracle (tests/golden/make_prism_field.py).
  256x256 Moho columns, 128x128 stations: the double and the mixed gradients
    of 0.5|gz - d|^2 with respect to depth and density against central
    differences (h = 1e-3 of a cell) at full size.
  32 line-search trials on the 256x256x64 mesh + 16 regional meshes of uneven
    size in one batched launch: every regional mesh and a set of trials
    against the plain double forward on a station subset.

TOLERANCES (written here): mixed vs double 1e-6 (normwise relative, the
precision target), also per station where the field is at least 10% of its
largest value (1e-5 where at least 1%: the error there is a few 1e-7 mGal);
plain double kernel vs the double oracle 1e-9 (two double summations of a
sum of 4e6 cancelling terms); gradients vs central differences 1e-5
(relative per entry)."""
import os

import numpy as np
import pytest

from helpers import rel_err
from ztm_gb300 import synth

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIELD = os.path.join(HERE, "golden", "prism_256x256x64_draped_fp64.npz")


def draped_inputs_and_fixture():
    if not os.path.exists(FIELD):
        pytest.skip("double field fixture not generated")
    mesh, rho, st = synth.draped_mesh_256x256x64()
    z = np.load(FIELD)
    # the fixture was computed from these inputs (fingerprints, not data)
    assert abs(float(np.sum(rho)) - float(z["rho_sum"])) <= 1e-9 * float(z["rho_abs_sum"])
    assert np.allclose(rho[::9973], z["rho_sample"], rtol=0, atol=1e-9)
    assert np.allclose(np.sum(st, axis=0), z["st_sum"], rtol=1e-12)
    return mesh, rho, st, z["gz"]


def test_draped_mesh_mixed_full_field(ctx):
    mesh, rho, st, ref = draped_inputs_and_fixture()
    out = ctx.prism(mesh, rho, st, precision="mixed")
    assert out.size == 16384
    assert rel_err(out, ref) <= 1e-6
    # per station: the error is absolute in nature (a few 1e-7 mGal), so the
    # relative bound holds where the station's field is not small
    rel = np.abs(out - ref) / np.abs(ref)
    assert np.max(rel[np.abs(ref) > 0.1 * np.abs(ref).max()]) <= 1e-6
    assert np.max(rel[np.abs(ref) > 0.01 * np.abs(ref).max()]) <= 1e-5


def test_draped_mesh_plain_double_full_field(ctx):
    mesh, rho, st, ref = draped_inputs_and_fixture()
    out = ctx.prism(mesh, rho, st, precision="fp64")
    assert rel_err(out, ref) <= 1e-9


def column_misfit_terms(ctx, im, depth, rho, st, data, c, which, h):
    """gz(+h) - gz(0) and gz(-h) - gz(0) of column c alone (the forward is a
    sum over columns, so a change of one column changes only its own term),
    in double, from one-column meshes at the column's cell."""
    ix, iy = c % im.nx, c // im.nx
    one = type(im)(1, 1, im.x0 + ix * im.dx, im.y0 + iy * im.dy, im.dx, im.dy, im.z_base)
    d0, r0 = np.array([depth[c]]), np.array([rho[c]])
    base = ctx.interface(one, d0, r0, st, precision="fp64")
    out = []
    for sgn in (1, -1):
        d1, r1 = d0.copy(), r0.copy()
        if which == "depth":
            d1[0] += sgn * h
        else:
            r1[0] += sgn * h
        out.append(ctx.interface(one, d1, r1, st, precision="fp64") - base)
    return out


def test_moho_columns_gradients_vs_central_differences_full_size(ctx):
    """256x256 Moho columns (depth 20-45 km), 128x128 stations, misfit
    0.5|gz - d|^2 with d the double forward of the true model plus 0.05 mGal
    noise, evaluated at the start model.  Central differences of step
    h = 1e-3 of a cell (1 m of depth; 1e-3 of |rho|) at five columns, two of
    them also through whole full-size double forwards."""
    im, depth_true, rho, st, start = synth.moho_columns()
    rng = np.random.default_rng(3)
    data = ctx.interface(im, depth_true, rho, st, precision="fp64") + rng.normal(0, 0.05, len(st))
    rng2 = np.random.default_rng(11)
    depth = start + rng2.normal(0.0, 2000.0, start.size)  # a model with structure
    m64, gz64, gr64, gd64 = ctx.interface_misfit(im, depth, rho, st, data, precision="fp64")
    mmx, gzmx, grmx, gdmx = ctx.interface_misfit(im, depth, rho, st, data, precision="mixed")
    r = gz64 - data
    cols = [int(c) for c in rng2.choice(depth.size, 5, replace=False)]
    for c in cols:
        for which, grad64, gradmx, h in (("depth", gd64, gdmx, 1.0),
                                         ("rho", gr64, grmx, 1e-3 * abs(rho[c]))):
            dp, dm = column_misfit_terms(ctx, im, depth, rho, st, data, c, which, h)
            fp = 0.5 * np.sum((r + dp) ** 2)
            fm = 0.5 * np.sum((r + dm) ** 2)
            fd = (fp - fm) / (2 * h)
            assert abs(grad64[c] - fd) <= 1e-5 * abs(fd), (which, c, grad64[c], fd)
            # the mixed gradient: 1e-5 of the entry, or of 1% of the largest
            # entry where the entry itself is small
            scale = max(abs(fd), 1e-2 * np.abs(grad64).max())
            assert abs(gradmx[c] - fd) <= 1e-5 * scale, (which, c, gradmx[c], fd)
    # two columns through whole full-size forwards in double
    for c in cols[:2]:
        e = np.zeros(depth.size)
        e[c] = 1.0
        fp = 0.5 * np.sum((ctx.interface(im, depth + e, rho, st, precision="fp64") - data) ** 2)
        fm = 0.5 * np.sum((ctx.interface(im, depth - e, rho, st, precision="fp64") - data) ** 2)
        fd = (fp - fm) / 2.0
        assert abs(gd64[c] - fd) <= 1e-4 * abs(fd), (c, gd64[c], fd)


def test_line_search_batch_against_double(ctx):
    """The batched launch of the line-search workload: each of the 16 regional
    meshes, and trials 0, 13 and 31 of the 256x256x64 mesh, against the
    plain double forward on a station subset."""
    jobs, alphas = synth.line_search_batch()
    outs = ctx.batch(jobs)
    mesh, trials, st = jobs[0]
    sub = np.arange(0, len(st), len(st) // 32)[:32]
    for k in (0, 13, 31):
        ref = ctx.prism(mesh, trials[k], st[sub], precision="fp64")
        assert rel_err(outs[0][k][sub], ref) <= 1e-6, k
    for j, (m, models, s) in enumerate(jobs[1:], start=1):
        sub = np.linspace(0, len(s) - 1, 48).astype(int)
        ref = ctx.prism(m, models[0], s[sub], precision="fp64")
        assert rel_err(outs[j][0][sub], ref) <= 1e-6, (j, m.nx, m.ny, m.nz, len(s))


def test_draped_mesh_linearity_and_adjoint_identity_full_size(ctx):
    """Size-independent properties at full size (256x256x64 prisms, 16,384
    stations), mixed method: the forward is linear in the density
    (gz(a r1 + b r2) = a gz(r1) + b gz(r2)) and the adjoint is its transpose
    (<w, F r> = <F^T w, r>), both to the precision target 1e-6."""
    mesh, rho, st = synth.draped_mesh_256x256x64()
    rng = np.random.default_rng(21)
    r2 = rng.normal(0.0, 100.0, rho.size)
    a, b = 0.7, -1.3
    g1 = ctx.prism(mesh, rho, st, precision="mixed")
    g2 = ctx.prism(mesh, r2, st, precision="mixed")
    g12 = ctx.prism(mesh, a * rho + b * r2, st, precision="mixed")
    assert rel_err(g12, a * g1 + b * g2) <= 1e-6
    w = rng.normal(0.0, 1.0, len(st))
    gt = ctx.adjoint(mesh, st, w, precision="mixed")
    lhs, rhs = float(np.dot(w, g1)), float(np.dot(gt, rho))
    assert abs(lhs - rhs) <= 1e-6 * float(np.sum(np.abs(w * g1)))


def test_pointmass_model_adjoint_identity_full_size(ctx):
    """The reference's point-mass model on the 256x256x64 geometry (its node
    grid, every node a station: 4.1e6 selected nodes x 65,536 stations): the
    float forward and the float transposed sum satisfy <w, J d> = <J^T w, d>
    to the float path's 1e-5."""
    mesh, rho, st = synth.draped_mesh_256x256x64()
    g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
    w = np.random.default_rng(22).normal(0.0, 1.0, g.di * g.dj)
    G = ctx.pointmass(g, drho, surf, precision="fp32")
    gt = ctx.pointmass_adjoint(g, surf, w, drho=drho, precision="fp32")
    lhs, rhs = float(np.dot(w, G)), float(np.dot(gt, drho))
    assert abs(lhs - rhs) <= 1e-5 * float(np.sum(np.abs(w * G)))
