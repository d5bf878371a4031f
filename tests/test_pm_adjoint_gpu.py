"""Derivatives of the reference's own gravity model on the GPU.

The reference builds the gravity columns of its Jacobian by forward
differences of whole forward runs (TFM.cpp:124-135).  The library gives them
analytically: the transposed point-mass sum (ztm_gfm_pointmass_adjoint), the
misfit of TFM.cpp:101-103 with its gradient (ztm_gfm_pointmass_misfit), and
the chain through the density builder of TFM.cpp:83-89
(ztm_gfm_pointmass_model_misfit).

TOLERANCES (written here, normwise relative unless stated):
  transposed sum vs the oracle's transposed TFM loop: 1e-12 double, 1e-5 float;
  dot-product identity <w, J drho> = <J^T w, drho>:    1e-12 double;
  misfit and residuals vs TFM.cpp:101-103 restated:   1e-12 double;
  gradients vs central finite differences:             1e-5 (relative per entry).
"""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import rel_err, tfm_density_inputs, tfm_like_inputs

pytestmark = pytest.mark.gpu

DIMS = [(21, 19, 9, 1, 2, 3), (16, 16, 9, 1, 3, 0), (13, 11, 7, 2, 2, 2), (61, 61, 33, 1, 2, 10)]


def interior_weights(grid, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(grid.di * grid.dj)
    b = grid.bfr
    m = np.zeros((grid.dj, grid.di), bool)
    m[b:grid.dj - b, b:grid.di - b] = True
    w[m.ravel()] = rng.normal(0.0, 1.0, int(m.sum()))
    return w, m.ravel()


@pytest.mark.parametrize("dims", DIMS)
def test_adjoint_matches_oracle(ctx, dims):
    """The transposed sum with a node list holding duplicates, with the
    threshold selection and over every node, double and float."""
    g = ztm_gb300.make_grid(*dims)
    drho, surf = tfm_like_inputs(*dims[:5], seed=dims[0] + 1)
    w, _ = interior_weights(g, 1)
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    nn = np.concatenate([nn, nn[::3]])
    # float: nodes at least one grid unit below the lowest station, as the
    # float forward's tests hold (every node of the grid includes nodes next
    # to the stations, where float keeps only a few digits)
    ii, jj = (dims[0] - 1) * dims[3] + 1, (dims[1] - 1) * dims[3] + 1
    k = (np.arange(drho.size) // (ii * jj)) / dims[4]
    deep = k <= surf.min() - 1.0
    for kw in ({"nn": nn}, {"drho": drho}, {}):
        ref = oracle.pointmass_adjoint(g, surf, w, **kw)
        out = ctx.pointmass_adjoint(g, surf, w, precision="fp64", **kw)
        assert rel_err(out, ref) <= 1e-12, kw.keys()
        out32 = ctx.pointmass_adjoint(g, surf, w, precision="fp32", **kw)
        assert rel_err(out32[deep], ref[deep]) <= 1e-5, kw.keys()
    sel = np.zeros(drho.size, bool)
    sel[nn] = True
    assert np.all(ctx.pointmass_adjoint(g, surf, w, nn=nn)[~sel] == 0.0)


@pytest.mark.parametrize("dims", DIMS)
def test_dot_product_identity(ctx, dims):
    """<w, J drho> = <J^T w, drho> with the GPU forward and adjoint."""
    g = ztm_gb300.make_grid(*dims)
    drho, surf = tfm_like_inputs(*dims[:5], seed=dims[0] + 2)
    w, m = interior_weights(g, 2)
    G = ctx.pointmass(g, drho, surf, precision="fp64")
    gt = ctx.pointmass_adjoint(g, surf, w, drho=drho, precision="fp64")
    lhs = float(np.dot(w[m], G[m]))
    rhs = float(np.dot(gt, drho))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), np.sum(np.abs(w[m] * G[m])))


def tfm_misfit(g, G, GD, g0, gsig):
    """TFM.cpp:101-103: y gets GD/gsig, f gets (G+g0)/gsig over the bfr
    interior, i outer and j inner; res = y - f, ssq = dot(res)."""
    res = []
    for i in range(g.bfr, g.di - g.bfr):
        for j in range(g.bfr, g.dj - g.bfr):
            n = i + j * g.di
            res.append(GD[n] / gsig - (G[n] + g0) / gsig)
    res = np.array(res)
    return float(np.dot(res, res)), res


@pytest.mark.parametrize("dims", [(21, 19, 9, 1, 2, 3), (61, 61, 33, 1, 2, 10)])
def test_misfit_reference_form(ctx, dims):
    g = ztm_gb300.make_grid(*dims)
    drho, surf = tfm_like_inputs(*dims[:5], seed=dims[0] + 3)
    rng = np.random.default_rng(3)
    G_ref = oracle.ref_tfm(g, drho, surf) if oracle.ref_tfm_available() else \
        oracle.pointmass_tfm(g, drho, surf)
    GD = G_ref + rng.normal(0, 0.5, G_ref.size) + 0.7
    g0, gsig = 0.4, 0.8
    ssq_ref, res_ref = tfm_misfit(g, G_ref, GD, g0, gsig)
    ssq, res, G, g_drho, g_g0 = ctx.pointmass_misfit(g, drho, surf, GD, g0, gsig)
    assert rel_err(G, G_ref) <= 1e-12
    assert rel_err(res, res_ref) <= 1e-12
    assert abs(ssq - ssq_ref) <= 1e-12 * ssq_ref
    assert abs(g_g0 - (-2.0 / gsig) * res_ref.sum()) <= 1e-12 * np.abs(res_ref).sum() * 2 / gsig
    # d ssq / d drho = J^T (-2 res / gsig) on the selected nodes
    w = np.zeros(g.di * g.dj)
    b = g.bfr
    idx = [i + j * g.di for i in range(b, g.di - b) for j in range(b, g.dj - b)]
    w[idx] = -2.0 * res_ref / gsig
    ref = oracle.pointmass_adjoint(g, surf, w, drho=drho)
    assert rel_err(g_drho, ref) <= 1e-12
    # float path
    ssq32, res32, _, g32, _ = ctx.pointmass_misfit(g, drho, surf, GD, g0, gsig, precision="fp32")
    # float forward: 1e-5 of the field's scale in each residual
    assert np.max(np.abs(res32 - res_ref)) <= 1e-5 * np.abs(G_ref).max() / gsig
    assert rel_err(g32, ref) <= 1e-4


def test_misfit_gradient_vs_finite_differences(ctx):
    dims = (21, 19, 9, 1, 2, 3)
    g = ztm_gb300.make_grid(*dims)
    drho, surf = tfm_like_inputs(*dims[:5], seed=7)
    GD = oracle.pointmass_tfm(g, drho * 1.1, surf) + 0.3
    _, _, _, grad, g_g0 = ctx.pointmass_misfit(g, drho, surf, GD, 0.2, 0.9)
    sel = np.nonzero(np.abs(drho) > 0.05)[0]
    rng = np.random.default_rng(0)
    for n in rng.choice(sel, 6, replace=False):
        h = 1e-4
        dp, dm = drho.copy(), drho.copy()
        dp[n] += h
        dm[n] -= h
        fp = ctx.pointmass_misfit(g, dp, surf, GD, 0.2, 0.9, gradient=False)[0]
        fm = ctx.pointmass_misfit(g, dm, surf, GD, 0.2, 0.9, gradient=False)[0]
        fd = (fp - fm) / (2 * h)
        assert abs(grad[n] - fd) <= 1e-5 * abs(fd), (n, grad[n], fd)
    h = 1e-4
    fp = ctx.pointmass_misfit(g, drho, surf, GD, 0.2 + h, 0.9, gradient=False)[0]
    fm = ctx.pointmass_misfit(g, drho, surf, GD, 0.2 - h, 0.9, gradient=False)[0]
    assert abs(g_g0 - (fp - fm) / (2 * h)) <= 1e-5 * abs(g_g0)


# ---- the chain through the density builder (TFM.cpp:83-89) ----------------
VM, RO, DR = 8.0, -0.4, 0.3


def model_case(di, dj, dk, seed):
    rc, sea, M, v = tfm_density_inputs(di, dj, dk, seed=seed)
    surf = sea + 0.3
    g = ztm_gb300.make_grid(di, dj, dk, 1, 2, 10 if di > 40 else 2)
    d_true = oracle.density_tfm(di, dj, dk, 1, 2, VM + 0.05, RO, DR, rc, sea, M + 0.2, v)
    GD = oracle.pointmass_tfm(g, d_true, surf) + 0.5
    return g, rc, sea, M, v, surf, GD


def selection(ctx, g, sea, M, v, vm, ro, dr, rc):
    d, _ = ctx.density(g.di, g.dj, g.dk, sea, M, v, vm, ro, dr, rc)
    return d != 0


def central_difference(ctx, g, rc, sea, M, v, surf, GD, which, idx=None, g0=0.3, gsig=0.7):
    """Central difference of ssq along one input, with a step that leaves the
    builder's node selection unchanged (the derivative is taken at fixed
    selection, as the analytic one is)."""
    base = dict(vm=VM, ro=RO, dr=DR, g0=g0)
    for h in (1e-5, 3e-6, 1e-6, 3e-7):
        vals = []
        sels = []
        for sgn in (1, -1):
            p = dict(base)
            Mx, vx = M, v
            if which in p:
                p[which] += sgn * h
            elif which == "M":
                Mx = M.copy()
                Mx[idx] += sgn * h
            else:
                vx = v.copy()
                vx[idx] += sgn * h
            r = ctx.pointmass_model_misfit(g, sea, Mx, vx, surf, GD, p["vm"], p["ro"], p["dr"], rc,
                                           g0=p["g0"], gsig=gsig, gradient=False)
            vals.append(r["ssq"])
            sels.append(selection(ctx, g, sea, Mx, vx, p["vm"], p["ro"], p["dr"], rc))
        if np.array_equal(sels[0], sels[1]):
            return (vals[0] - vals[1]) / (2 * h)
    return None  # every step moved a node across the selection threshold


@pytest.mark.parametrize("di,dj,dk", [(21, 19, 13), (61, 61, 33)])
def test_model_gradient_vs_finite_differences(ctx, di, dj, dk):
    g, rc, sea, M, v, surf, GD = model_case(di, dj, dk, seed=di + 4)
    r = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7)
    gp = r["g_par"]
    checked = 0
    for k, name in enumerate(("vm", "ro", "dr", "g0")):
        fd = central_difference(ctx, g, rc, sea, M, v, surf, GD, name)
        if fd is None:
            continue
        assert abs(gp[k] - fd) <= 1e-5 * abs(fd), (name, gp[k], fd)
        checked += 1
    # Moho nodes where the gradient is largest (blend zones above selected
    # nodes), and velocity nodes
    for idx in np.argsort(-np.abs(r["g_M"]))[:4]:
        fd = central_difference(ctx, g, rc, sea, M, v, surf, GD, "M", int(idx))
        if fd is None:
            continue
        assert abs(r["g_M"][idx] - fd) <= 1e-5 * abs(fd), ("M", idx, r["g_M"][idx], fd)
        checked += 1
    for idx in np.argsort(-np.abs(r["g_v"]))[:4]:
        fd = central_difference(ctx, g, rc, sea, M, v, surf, GD, "v", int(idx))
        if fd is None:
            continue
        assert abs(r["g_v"][idx] - fd) <= 1e-5 * abs(fd), ("v", idx, r["g_v"][idx], fd)
        checked += 1
    # a global parameter moves every node's density, so a step can cross the
    # selection threshold of one of ~1e5 nodes; all but a few entries must be
    # checkable
    assert checked >= 9, checked


def test_model_misfit_matches_oracle_chain(ctx):
    """ssq, res and G of the chained call against the oracle's builder and
    TFM loop, and d ssq / d M against central differences of the oracle
    chain itself (no GPU in the differences)."""
    di, dj, dk = 21, 19, 13
    g, rc, sea, M, v, surf, GD = model_case(di, dj, dk, seed=3)
    r = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7)

    def ora(Mx):
        d = oracle.density_tfm(di, dj, dk, 1, 2, VM, RO, DR, rc, sea, Mx, v)
        G = oracle.pointmass_tfm(g, d, surf)
        return tfm_misfit(g, G, GD, 0.3, 0.7), d, G

    (ssq, res), d0, G0 = ora(M)
    assert rel_err(r["G"], G0) <= 1e-12
    assert rel_err(r["res"], res) <= 1e-12
    assert abs(r["ssq"] - ssq) <= 1e-12 * ssq
    for idx in np.argsort(-np.abs(r["g_M"]))[:3]:
        h = 1e-6
        Mp, Mm = M.copy(), M.copy()
        Mp[idx] += h
        Mm[idx] -= h
        (sp, _), dp, _ = ora(Mp)
        (sm, _), dm, _ = ora(Mm)
        if not np.array_equal(dp != 0, dm != 0):
            continue
        fd = (sp - sm) / (2 * h)
        assert abs(r["g_M"][idx] - fd) <= 1e-5 * abs(fd)


def test_model_misfit_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    g, rc, sea, M, v, surf, GD = model_case(21, 19, 13, seed=9)
    host = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7)
    d = lambda a: torch.tensor(a, device="cuda")
    dev = ctx.pointmass_model_misfit(g, d(sea), d(M), d(v), d(surf), d(GD), VM, RO, DR, rc,
                                     g0=0.3, gsig=0.7)
    ctx.sync()
    assert float(dev["ssq"].item()) == host["ssq"]
    for k in ("res", "G", "g_par"):
        assert np.array_equal(dev[k].cpu().numpy(), host[k]), k
    # atomics in the builder's adjoint: the same up to the order of the adds
    for k in ("g_M", "g_v"):
        assert rel_err(dev[k].cpu().numpy(), host[k]) <= 1e-13, k


def test_edge_cases_no_interior_and_no_gradient(ctx):
    """bfr leaving no interior station: the transposed sum is zero and the
    misfit is zero; the misfit without its gradient returns the same ssq and
    residual as with it."""
    g = ztm_gb300.make_grid(8, 8, 4, 1, 2, 4)
    drho, surf = tfm_like_inputs(8, 8, 4, seed=6)
    w = np.ones(64)
    assert np.all(ctx.pointmass_adjoint(g, surf, w, drho=drho) == 0.0)
    ssq, res, G, gd, g0 = ctx.pointmass_misfit(g, drho, surf, np.ones(64), 0.1, 1.0)
    assert ssq == 0.0 and res.size == 0 and np.all(G == 0.0) and np.all(gd == 0.0)
    assert g0 == 0.0
    g = ztm_gb300.make_grid(21, 19, 9, 1, 2, 3)
    drho, surf = tfm_like_inputs(21, 19, 9, seed=8)
    GD = oracle.pointmass_tfm(g, drho, surf) + 0.2
    a = ctx.pointmass_misfit(g, drho, surf, GD, 0.1, 0.5)
    b = ctx.pointmass_misfit(g, drho, surf, GD, 0.1, 0.5, gradient=False)
    assert a[0] == b[0] and np.array_equal(a[1], b[1]) and b[3] is None


def test_model_misfit_without_gradient(ctx):
    g, rc, sea, M, v, surf, GD = model_case(21, 19, 13, seed=12)
    a = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7)
    b = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7,
                                   gradient=False)
    assert a["ssq"] == b["ssq"] and np.array_equal(a["G"], b["G"]) and "g_M" not in b


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_model_misfit_field_is_the_model_forward(ctx, precision):
    """The chained call's G is ztm_gfm_pointmass_model's field, bit for bit,
    so the central differences above are differences of that forward."""
    g, rc, sea, M, v, surf, GD = model_case(61, 61, 33, seed=5)
    r = ctx.pointmass_model_misfit(g, sea, M, v, surf, GD, VM, RO, DR, rc, g0=0.3, gsig=0.7,
                                   precision=precision)
    G = ctx.pointmass_model(g, sea, M, v, surf, VM, RO, DR, rc, precision=precision)
    assert np.array_equal(r["G"], G)
