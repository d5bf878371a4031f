"""Pins of the CPU oracle (no GPU).  The reference has no tests and no
golden outputs; the oracle is pinned by (a) agreement of the two restated
point-mass paths and by the reference GF kernel's own outputs
(tests/golden, made on a GPU by tests/golden/make_golden.py), and (b)
mathematical known answers for the prism model, which has no reference
implementation."""
import math
import os

import numpy as np
import pytest

import oracle
import ztm_gb300
from helpers import rel_err, small_mesh, tfm_like_inputs

G = 6.67e-11
HERE = os.path.dirname(os.path.abspath(__file__))


# ---- point-mass model (TFM.cpp:95-99, GFM_GPU.cu:16-22) --------------------
# The reference GF kernel accumulates in float without compensation, in the
# order its atomics land; with mixed-sign densities the sums cancel, so its
# outputs carry up to ~1e-5 normwise error (measured 1e-6..1e-5 on the
# golden cases).  TOL_GF bounds that.
TOL_GF = 5e-5


def test_tfm_and_gf_restatements_agree():
    g = ztm_gb300.make_grid(21, 19, 9, 1, 2, 3)
    drho, surf = tfm_like_inputs(21, 19, 9, seed=11)
    a = oracle.pointmass_tfm(g, drho, surf)
    b = oracle.pointmass_gf(g, drho.astype(np.float32), surf.astype(np.float32))
    assert rel_err(b, a) <= TOL_GF


def test_tfm_single_node_by_hand():
    g = ztm_gb300.make_grid(5, 5, 3, 1, 2, 1)
    ii, jj, kk = 5, 5, 5
    drho = np.zeros(ii * jj * kk)
    n = 2 + 3 * ii + 1 * ii * jj  # i=2, j=3, k=0.5
    drho[n] = 0.3
    surf = np.full(25, 2.25)
    G_ = oracle.pointmass_tfm(g, drho, surf)
    i0, j0 = 1, 2
    d2 = (i0 - 2) ** 2 + (j0 - 3) ** 2 + (2.25 - 0.5) ** 2
    want = 66.7 * 0.3 * (2.25 - 0.5) / d2 ** 1.5 / 2
    assert G_[i0 + 5 * j0] == pytest.approx(want, rel=1e-15)
    assert G_[0] == 0.0  # buffer stations untouched


def test_tfm_threshold_selects_like_nn():
    g = ztm_gb300.make_grid(11, 11, 5, 1, 2, 2)
    drho, surf = tfm_like_inputs(11, 11, 5, seed=12)
    nn = np.nonzero(np.abs(drho) > 0.001)[0]
    assert np.array_equal(oracle.pointmass_tfm(g, drho, surf),
                          oracle.pointmass_tfm(g, drho, surf, nn=nn))


@pytest.mark.skipif(not oracle.ref_tfm_available(), reason="reference TFM.cpp lambda not built")
@pytest.mark.parametrize("dims", [(21, 19, 9, 1, 2, 3), (61, 61, 33, 1, 2, 10), (16, 16, 9, 1, 3, 0),
                                  (31, 29, 17, 2, 2, 5), (5, 5, 2, 1, 1, 0)])
def test_restatement_equals_reference_lambda(dims):
    """The restatement of TFM.cpp:95-99 against the reference's own lambda,
    cut verbatim out of TFM.cpp and compiled (oracle/build.py): bit for bit,
    with the threshold list and with a list holding duplicates."""
    di, dj, dk, fh, fv, bfr = dims
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
    drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=di + dk)
    assert np.array_equal(oracle.ref_tfm(g, drho, surf), oracle.pointmass_tfm(g, drho, surf))
    nn = np.nonzero(np.abs(drho) > 0.05)[0].astype(np.int32)
    nn = np.concatenate([nn, nn[::5]])
    assert np.array_equal(oracle.ref_tfm(g, drho, surf, nn=nn),
                          oracle.pointmass_tfm(g, drho, surf, nn=nn))


@pytest.mark.skipif(not oracle.ref_tfm_available(), reason="reference TFM.cpp lambda not built")
def test_reference_lambda_rows_sample_matches_full():
    """The row-range entry (the bench's bounded sample) is the same lambda."""
    g = ztm_gb300.make_grid(31, 29, 17, 1, 2, 5)
    drho, surf = tfm_like_inputs(31, 29, 17, seed=9)
    full = oracle.ref_tfm(g, drho, surf).reshape(29, 31)
    part, _ = oracle.ref_tfm_rows(g, drho, surf, 7, 12)
    part = part.reshape(29, 31)
    assert np.array_equal(part[7:12], full[7:12])
    assert np.all(part[:7] == 0) and np.all(part[12:] == 0)


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(os.path.join(HERE, "golden"))
                                        if f.startswith("gf_") and f.endswith(".npz")))
def test_golden_reference_gf_outputs(name):
    """Outputs of the unchanged reference GF kernel (float, atomics) on
    seeded inputs vs the double restatement of TFM.cpp:95-99."""
    z = np.load(os.path.join(HERE, "golden", name))
    di, dj, dk, fh, fv, bfr = (int(v) for v in z["dims"])
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
    ref = oracle.pointmass_tfm(g, z["drho"].astype(np.float64), z["surf"].astype(np.float64))
    assert rel_err(z["g"], ref) <= TOL_GF
    gf = oracle.pointmass_gf(g, z["drho"], z["surf"])
    assert rel_err(z["g"], gf) <= TOL_GF


# ---- prism model: known answers --------------------------------------------
def test_prism_matches_numerical_quadrature():
    integrate = pytest.importorskip("scipy.integrate")
    for case in [(0, 0, 1, -1, 1, -1, 1, -2, -1), (0.3, -2, 0.5, -1, 2, -1, 1.5, -3, -0.5),
                 (5, 4, 3, 0, 1, 0, 1, -1, 0)]:
        xs, ys, zs, X1, X2, Y1, Y2, Z1, Z2 = case
        f = lambda z, y, x: (zs - z) / ((x - xs) ** 2 + (y - ys) ** 2 + (zs - z) ** 2) ** 1.5
        num = integrate.tplquad(f, X1, X2, Y1, Y2, Z1, Z2, epsabs=1e-12, epsrel=1e-10)[0]
        assert oracle.prism_unit(*case) == pytest.approx(num, rel=1e-8)


def test_face_matches_numerical_quadrature():
    integrate = pytest.importorskip("scipy.integrate")
    for xs, ys, zs, x0, x1, y0, y1, zf in [(0, 0, 1, -1, 1, -1, 1, 0), (0.5, 3, 2, -1, 2, 0, 1, 0),
                                           (0, 0, -1.5, -1, 1, -2, 1, 0)]:
        w = zs - zf
        f = lambda y, x: w / ((x - xs) ** 2 + (y - ys) ** 2 + w * w) ** 1.5
        num = integrate.dblquad(f, x0, x1, y0, y1, epsabs=1e-13)[0]
        assert oracle.face_unit(xs, ys, zs, x0, x1, y0, y1, zf) == pytest.approx(num, rel=1e-9)


def test_bouguer_slab_limit():
    a, t = 1.0e7, 100.0  # half width 10^4 km, 100 m thick, station on top
    u = oracle.prism_unit(0, 0, 0, -a, a, -a, a, -t, 0)
    assert u == pytest.approx(2 * math.pi * t, rel=1e-4)


def test_superposition_of_eight_subprisms():
    xs, ys, zs = 1234.0, -567.0, 890.0
    x0, x1, y0, y1, z0, z1 = -1000.0, 3000.0, -2000.0, 500.0, -4000.0, -300.0
    whole = oracle.prism_unit(xs, ys, zs, x0, x1, y0, y1, z0, z1)
    xm, ym, zm = 0.5 * (x0 + x1), 0.5 * (y0 + y1), 0.5 * (z0 + z1)
    parts = 0.0
    for xa, xb in ((x0, xm), (xm, x1)):
        for ya, yb in ((y0, ym), (ym, y1)):
            for za, zb in ((z0, zm), (zm, z1)):
                parts += oracle.prism_unit(xs, ys, zs, xa, xb, ya, yb, za, zb)
    assert parts == pytest.approx(whole, rel=1e-12)


def test_reflection_antisymmetry():
    b = oracle.prism_unit(0.3, 0.2, 0.0, -1, 2, -1.5, 1, -3, -1)
    a = oracle.prism_unit(0.3, 0.2, 0.0, -1, 2, -1.5, 1, 1, 3)
    assert a == pytest.approx(-b, rel=1e-13)


def test_far_field_point_mass_limit():
    dx, dy, dz = 1000.0, 800.0, 500.0
    V = dx * dy * dz
    for R in (2e4, 1e5, 5e5):
        zs = R
        u = oracle.prism_unit(0.3 * R, 0.1 * R, zs, -dx / 2, dx / 2, -dy / 2, dy / 2, -dz / 2, dz / 2)
        X, Y, Z = 0.3 * R, 0.1 * R, zs
        r = math.sqrt(X * X + Y * Y + Z * Z)
        pm = V * Z / r ** 3
        assert abs(u - pm) / pm <= 0.5 * (dx / r) ** 2


def test_far_field_ties_prism_model_to_reference_point_mass_model():
    """The reference's point-mass model (TFM.cpp:95-99, node-centred cells,
    66.7 = G*h for h = 10 km) is the far-field limit of the prism model."""
    h_km = 10.0
    di = dj = 7
    dk = 4
    fh, fv = 1, 2
    g = ztm_gb300.make_grid(di, dj, dk, fh, fv, 0)
    ii, jj, kk = di, dj, (dk - 1) * fv + 1
    rng = np.random.default_rng(3)
    drho = rng.uniform(0.05, 0.3, ii * jj * kk)  # g/cc
    surf = np.full(di * dj, 60.0)  # 600 km above the nodes
    pm = oracle.pointmass_tfm(g, drho, surf)
    # the same masses as prisms of h x h x h/fv centred on the nodes (metres)
    h = h_km * 1000.0
    geom, rho = [], []
    for n in range(ii * jj * kk):
        i, j, k = n % ii, (n // ii) % jj, n // (ii * jj)
        xc, yc, zc = i * h, j * h, k * h / fv
        geom.append((xc - h / 2, xc + h / 2, yc - h / 2, yc + h / 2, zc - h / (2 * fv),
                     zc + h / (2 * fv)))
        rho.append(drho[n] * 1000.0)
    st = np.array([(i0 * h, j0 * h, 60.0 * h) for j0 in range(dj) for i0 in range(di)])
    pr = oracle.prism_list(np.array(geom), np.array(rho), st, G=G)
    assert rel_err(pr, pm) <= 1e-4


def test_face_is_derivative_of_prism_in_top():
    xs, ys, zs = 300.0, -200.0, 150.0
    x0, x1, y0, y1, zb, zt = -1000.0, 800.0, -600.0, 900.0, -5000.0, -2000.0
    hstep = 1e-3 * 1000.0
    up = oracle.prism_unit(xs, ys, zs, x0, x1, y0, y1, zb, zt + hstep)
    dn = oracle.prism_unit(xs, ys, zs, x0, x1, y0, y1, zb, zt - hstep)
    fd = (up - dn) / (2 * hstep)
    assert oracle.face_unit(xs, ys, zs, x0, x1, y0, y1, zt) == pytest.approx(fd, rel=1e-6)


def test_long_double_agrees_with_double():
    mesh, rho = small_mesh(6, 5, 4, seed=2)
    st = np.array([[500.0, 2500.0, 800.0], [-2000.0, 3000.0, 250.0], [1e5, 1e5, 10.0]])
    a = oracle.prism_mesh(mesh, rho, st)
    b = oracle.prism_mesh(mesh, rho, st, long_double=True)
    assert rel_err(a, b) <= 1e-11


def test_mesh_equals_list():
    mesh, rho = small_mesh(5, 4, 3, seed=4)
    st = np.array([[100.0, 2000.0, 300.0], [4000.0, -1000.0, 50.0]])
    geom = []
    for l in range(mesh.nz):
        for iy in range(mesh.ny):
            for ix in range(mesh.nx):
                geom.append((mesh.x0 + ix * mesh.dx, mesh.x0 + (ix + 1) * mesh.dx,
                             mesh.y0 + iy * mesh.dy, mesh.y0 + (iy + 1) * mesh.dy,
                             mesh.z_top - (l + 1) * mesh.dz, mesh.z_top - l * mesh.dz))
    assert rel_err(oracle.prism_list(np.array(geom), rho, st), oracle.prism_mesh(mesh, rho, st)) <= 1e-14


# ---- adjoints of the oracle are exact transposes / derivatives --------------
def test_mesh_adjoint_dot_product():
    mesh, rho = small_mesh(5, 4, 3, seed=5)
    rng = np.random.default_rng(0)
    st = np.stack([rng.uniform(-4000, 3000, 9), rng.uniform(1000, 5000, 9), rng.uniform(250, 900, 9)], 1)
    r = rng.normal(size=9)
    dr = rng.normal(size=rho.size)
    lhs = np.dot(oracle.mesh_adjoint(mesh, st, r), dr)
    rhs = np.dot(r, oracle.prism_mesh(mesh, dr, st))
    assert lhs == pytest.approx(rhs, rel=1e-12)


def test_interface_adjoint_against_central_differences():
    im = ztm_gb300.make_imesh(6, 5, 1000.0, 1000.0, -8000.0)
    rng = np.random.default_rng(1)
    depth = rng.uniform(2000.0, 6000.0, 30)
    rho = np.full(30, -400.0)
    st = np.stack([rng.uniform(0, 6000, 7), rng.uniform(0, 5000, 7), np.zeros(7)], 1)
    data = oracle.interface_fwd(im, depth + 300.0, rho, st)
    res = oracle.interface_fwd(im, depth, rho, st) - data
    g_rho, g_dep = oracle.interface_adj(im, depth, rho, st, res)

    def misfit(d, r_):
        return 0.5 * np.sum((oracle.interface_fwd(im, d, r_, st) - data) ** 2)

    h = 1e-3 * 1000.0  # 1 m
    for c in (0, 7, 29):
        e = np.zeros(30)
        e[c] = h
        fd = (misfit(depth + e, rho) - misfit(depth - e, rho)) / (2 * h)
        assert g_dep[c] == pytest.approx(fd, rel=1e-5)
        e = np.zeros(30)
        e[c] = 1.0
        fd = (misfit(depth, rho + e) - misfit(depth, rho - e)) / 2.0
        assert g_rho[c] == pytest.approx(fd, rel=1e-6)


# ---- density builder (TFM.cpp:85-89) ---------------------------------------
def test_density_builder_by_hand():
    from helpers import tfm_density_inputs
    rc, sea, M, v = tfm_density_inputs(21, 19, 13, seed=1)
    di, dj, dk, fh, fv = 21, 19, 13, 1, 2
    vm, ro, dr = 8.0, -0.4, 0.3
    d = oracle.density_tfm(di, dj, dk, fh, fv, vm, ro, dr, rc, sea, M, v)
    ii, jj, kk = di, dj, (dk - 1) * fv + 1
    assert d.size == ii * jj * kk
    # a node far above both Mohos: r0 = r1 = ro -> not selected
    n_top = 5 + 7 * ii + (kk - 1) * ii * jj
    assert d[n_top] == 0.0
    # a node between the two Mohos is selected when deep enough and the
    # contrast exceeds 0.001
    sel = np.count_nonzero(d)
    assert 0 < sel < d.size
    # by hand for one node below both Mohos: r0 = 0, r1 = dr*(v-vm)
    i, j, kf = 10, 9, 4  # k = 2.0 grid units, far below the Moho (~6.5)
    n = i + j * ii + kf * ii * jj
    k = kf / fv
    vv = v.reshape(dk, dj, di)[int(k), j, i]  # k integer: the node value itself
    r1 = dr * (vv - vm)
    assert d[n] == (r1 if abs(r1) > 0.001 else 0.0)
