"""Adjoint kernels on the GPU: against the double oracle, the dot-product
test, central finite differences (h = 1e-3 in units of the cell) and
torch.autograd.gradcheck through the autograd wrapper.

TOLERANCES: FP64 kernels vs oracle 1e-10; mixed vs FP64 1e-6 (normwise);
gradient vs central differences 1e-5 (relative)."""
import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import rel_err, small_mesh

pytestmark = pytest.mark.gpu


def stations_over(mesh, n, seed, zmin=1.0, zmax=3000.0):
    rng = np.random.default_rng(seed)
    X1 = mesh.x0 + mesh.nx * mesh.dx
    Y1 = mesh.y0 + mesh.ny * mesh.dy
    return np.stack([rng.uniform(mesh.x0 - 1000, X1 + 1000, n),
                     rng.uniform(mesh.y0 - 1000, Y1 + 1000, n),
                     rng.uniform(mesh.z_top + zmin, mesh.z_top + zmax, n)], 1)


@pytest.mark.parametrize("shape", [(12, 10, 6), (40, 32, 12)])
def test_mesh_adjoint_vs_oracle(ctx, shape):
    mesh, _ = small_mesh(*shape, seed=1)
    st = stations_over(mesh, 50, 2)
    r = np.random.default_rng(3).normal(size=50)
    ref = oracle.mesh_adjoint(mesh, st, r)
    assert rel_err(ctx.adjoint(mesh, st, r, precision="fp64"), ref) <= 1e-10
    assert rel_err(ctx.adjoint(mesh, st, r, precision="mixed"), ref) <= 1e-6


def test_mesh_adjoint_dot_product(ctx):
    mesh, rho = small_mesh(48, 40, 10, seed=4)
    st = stations_over(mesh, 200, 5)
    rng = np.random.default_rng(6)
    r = rng.normal(size=200)
    for p in ("fp64", "mixed"):
        lhs = np.dot(ctx.adjoint(mesh, st, r, precision=p), rho)
        rhs = np.dot(r, ctx.prism(mesh, rho, st, precision=p))
        # double: forward and adjoint sum the cancelling corner terms by
        # vertices in different orders (1e-10, the double kernels' tolerance
        # against the oracle)
        assert lhs == pytest.approx(rhs, rel=1e-6 if p == "mixed" else 1e-10)


def iface_case(n=24, seed=0, ns=60):
    rng = np.random.default_rng(seed)
    im = ztm_gb300.make_imesh(n, n - 3, 1000.0, 1000.0, -30000.0, x0=-2000.0, y0=500.0)
    nc = n * (n - 3)
    depth = rng.uniform(3000.0, 25000.0, nc)
    rho = rng.uniform(-450.0, -350.0, nc)
    st = np.stack([rng.uniform(-5000, n * 1000.0, ns), rng.uniform(0, (n - 3) * 1000.0, ns),
                   rng.uniform(0.0, 1500.0, ns)], 1)
    return im, depth, rho, st


def test_interface_forward_vs_oracle(ctx):
    im, depth, rho, st = iface_case()
    ref = oracle.interface_fwd(im, depth, rho, st)
    assert rel_err(ctx.interface(im, depth, rho, st, precision="fp64"), ref) <= 1e-10
    assert rel_err(ctx.interface(im, depth, rho, st, precision="mixed"), ref) <= 1e-6


def test_interface_adjoint_vs_oracle(ctx):
    im, depth, rho, st = iface_case(seed=1)
    r = np.random.default_rng(2).normal(size=len(st))
    gr, gd = oracle.interface_adj(im, depth, rho, st, r)
    for p, tol in (("fp64", 1e-10), ("mixed", 1e-6)):
        a, b = ctx.interface_adjoint(im, depth, rho, st, r, precision=p)
        assert rel_err(a, gr) <= tol
        assert rel_err(b, gd) <= tol


def test_interface_misfit_gradient_vs_central_differences(ctx):
    im, depth, rho, st = iface_case(n=16, seed=3, ns=40)
    data = oracle.interface_fwd(im, depth + 500.0 * np.sin(np.arange(depth.size)), rho, st)
    mis, gz, gr, gd = ctx.interface_misfit(im, depth, rho, st, data, precision="fp64")
    assert rel_err(gz, oracle.interface_fwd(im, depth, rho, st)) <= 1e-10
    assert mis == pytest.approx(0.5 * np.sum((gz - data) ** 2), rel=1e-12)
    h = 1e-3 * im.dx  # h = 1e-3 cell
    for c in (0, 37, depth.size - 1):
        e = np.zeros(depth.size)
        e[c] = h
        mp = ctx.interface_misfit(im, depth + e, rho, st, data, precision="fp64")[0]
        mm = ctx.interface_misfit(im, depth - e, rho, st, data, precision="fp64")[0]
        assert gd[c] == pytest.approx((mp - mm) / (2 * h), rel=1e-5)
    mis_m, gz_m, gr_m, gd_m = ctx.interface_misfit(im, depth, rho, st, data, precision="mixed")
    assert rel_err(gz_m, gz) <= 1e-6
    # the gradient is linear in the residual gz - data, whose relative error
    # is the forward's scaled by max|gz| / max|gz - data|
    amp = np.max(np.abs(gz)) / np.max(np.abs(gz - data))
    assert rel_err(gd_m, gd) <= 1e-6 * (1 + amp) and rel_err(gr_m, gr) <= 1e-6 * (1 + amp)


def test_moho_256_gradients_mixed_vs_fp64(ctx):
    """256x256 Moho columns, 128x128 stations: mixed vs double
    gradients and the misfit, full size."""
    from ztm_gb300 import synth
    im, depth, rho, st, start = synth.moho_columns()
    rng = np.random.default_rng(3)
    data = ctx.interface(im, depth, rho, st, precision="fp64") + rng.normal(0, 0.05, len(st))
    m64 = ctx.interface_misfit(im, start, rho, st, data, precision="fp64")
    mmx = ctx.interface_misfit(im, start, rho, st, data, precision="mixed")
    assert mmx[0] == pytest.approx(m64[0], rel=1e-6)
    assert rel_err(mmx[1], m64[1]) <= 1e-6
    assert rel_err(mmx[2], m64[2]) <= 1e-6
    assert rel_err(mmx[3], m64[3]) <= 1e-6


def test_autograd_gradcheck(ctx):
    torch = pytest.importorskip("torch")
    from ztm_gb300.autograd import InterfaceGravity, PrismGravity
    mesh, rho = small_mesh(6, 5, 4, seed=7)
    st = torch.tensor(stations_over(mesh, 8, 8), device="cuda")
    r = torch.tensor(rho / 100.0, device="cuda", requires_grad=True)
    f = lambda x: PrismGravity.apply(x * 100.0, ctx, mesh, st, "fp64")
    assert torch.autograd.gradcheck(f, (r,), eps=1e-3, atol=1e-8, rtol=1e-5)
    im, depth, rhoc, sti = iface_case(n=6, seed=9, ns=10)
    d = torch.tensor(depth / 1000.0, device="cuda", requires_grad=True)
    rc = torch.tensor(rhoc / 100.0, device="cuda", requires_grad=True)
    sti = torch.tensor(sti, device="cuda")
    g = lambda dd, rr: InterfaceGravity.apply(dd * 1000.0, rr * 100.0, ctx, im, sti, "fp64")
    assert torch.autograd.gradcheck(g, (d, rc), eps=1e-3, atol=1e-8, rtol=1e-5)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_interface_depth_jvp_dot_product_and_differences(ctx, precision, tol):
    """J v from ztm_gfm_interface_jvp against the depth adjoint (J^T w) by the
    dot-product identity, and against central differences of the forward."""
    from ztm_gb300 import synth
    im, depth, rho, st, _ = synth.moho_columns(seed=8, n=48, ns_side=24, cell=1000.0)
    rng = np.random.default_rng(9)
    v = rng.normal(0.0, 100.0, depth.size)
    w = rng.normal(0.0, 1.0, len(st))
    jv = ctx.interface_jvp(im, depth, rho, st, v, precision=precision)
    _, jtw = ctx.interface_adjoint(im, depth, rho, st, w, precision=precision)
    lhs, rhs = float(np.dot(jv, w)), float(np.dot(v, jtw))
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs))
    if precision == "fp64":
        h = 1e-3
        fd = (ctx.interface(im, depth + h * v, rho, st, precision="fp64") -
              ctx.interface(im, depth - h * v, rho, st, precision="fp64")) / (2 * h)
        assert rel_err(jv, fd) <= 1e-5
    else:
        ref = ctx.interface_jvp(im, depth, rho, st, v, precision="fp64")
        assert rel_err(jv, ref) <= 1e-6
