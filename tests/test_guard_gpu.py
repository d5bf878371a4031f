"""Outputs written in place: every output array of a call is the interior of
a larger buffer whose guard bands hold a marker bit pattern; the call must
write the interior (no marker left there) and nothing outside it, for device
arrays (ZTM_FLAG_DEVICE_PTRS) and for host arrays."""
import ctypes

import numpy as np
import pytest

import ztm_gb300
from ztm_gb300 import _lib
from helpers import awkward_stations, small_mesh

pytestmark = pytest.mark.gpu
GUARD = 4096                      # doubles on each side of an output
MARK = np.int64(0x7FF8DEAD0000BEEF)  # a NaN with a payload no result can have


def _host_buf(n):
    b = np.empty(n + 2 * GUARD, dtype=np.float64)
    b.view(np.int64)[:] = MARK
    return b


def _dev_buf(n):
    import torch
    return torch.from_numpy(_host_buf(n)).cuda()


def _check(bits, n):
    bits = np.asarray(bits).view(np.int64)
    assert np.all(bits[:GUARD] == MARK), "written before the output"
    assert np.all(bits[GUARD + n:] == MARK), "written past the output"
    assert not np.any(bits[GUARD:GUARD + n] == MARK), "output not written"


def _opts(precision, device):
    return _lib.Opts(precision, _lib.FLAG_DEVICE_PTRS if device else 0, 0.0, 0.0, 0, 0)


@pytest.mark.parametrize("device", [True, False])
@pytest.mark.parametrize("precision", [ztm_gb300.PREC_MIXED, ztm_gb300.PREC_FP64])
def test_prism_forward_and_adjoint_stay_inside_their_outputs(ctx, device, precision):
    import torch
    mesh, rho = small_mesh(37, 29, 11, seed=12)
    st = awkward_stations(mesh, n_random=150)
    ns, npr = len(st), mesh.nx * mesh.ny * mesh.nz
    res = np.random.default_rng(3).normal(0.0, 1.0, ns)
    if device:
        d_rho, d_st, d_res = (torch.tensor(x, device="cuda") for x in (rho, st.ravel(), res))
        gz, g = _dev_buf(ns), _dev_buf(npr)
        ptr = lambda t, off=0: ctypes.c_void_p(t.data_ptr() + 8 * off)
        args_f = (ptr(d_rho), ns, ptr(d_st), ptr(gz, GUARD))
        args_a = (ns, ptr(d_st), ptr(d_res), ptr(g, GUARD))
    else:
        gz, g = _host_buf(ns), _host_buf(npr)
        ptr = lambda a, off=0: ctypes.c_void_p(a.ctypes.data + 8 * off)
        st_c = np.ascontiguousarray(st.ravel())
        args_f = (ptr(rho), ns, ptr(st_c), ptr(gz, GUARD))
        args_a = (ns, ptr(st_c), ptr(res), ptr(g, GUARD))
    o = _opts(precision, device)
    assert ctx._lib.ztm_gfm_prism(ctx._h, ctypes.byref(mesh), *args_f, ctypes.byref(o)) == 0
    assert ctx._lib.ztm_gfm_adjoint(ctx._h, ctypes.byref(mesh), *args_a, ctypes.byref(o)) == 0
    ctx.sync()
    if device:
        torch.cuda.synchronize()
        gz, g = gz.cpu().numpy(), g.cpu().numpy()
    _check(gz, ns)
    _check(g, npr)
    # the interior is the field itself
    ref = ctx.prism(mesh, rho, st, precision="mixed" if precision == ztm_gb300.PREC_MIXED
                    else "fp64")
    np.testing.assert_array_equal(gz[GUARD:GUARD + ns], ref)


def test_batch_stays_inside_its_outputs(ctx):
    import torch
    jobs = []
    outs = []
    for i, (shape, nm) in enumerate((((24, 20, 9), 3), ((17, 13, 8), 1))):
        mesh, rho = small_mesh(*shape, seed=20 + i)
        st = awkward_stations(mesh, n_random=70 + 30 * i, seed=i)
        trials = np.stack([rho * (1.0 + 0.1 * m) for m in range(nm)])
        n = nm * len(st)
        buf = _dev_buf(n)
        d_r = torch.tensor(trials.ravel(), device="cuda")
        d_s = torch.tensor(st.ravel(), device="cuda")
        jobs.append(_lib.Job(mesh, nm, ctypes.c_void_p(d_r.data_ptr()), len(st),
                             ctypes.c_void_p(d_s.data_ptr()),
                             ctypes.c_void_p(buf.data_ptr() + 8 * GUARD)))
        outs.append((buf, n, d_r, d_s))
    arr = (_lib.Job * len(jobs))(*jobs)
    o = _opts(ztm_gb300.PREC_MIXED, True)
    assert ctx._lib.ztm_gfm_batch(ctx._h, arr, len(jobs), ctypes.byref(o)) == 0
    ctx.sync()
    torch.cuda.synchronize()
    for buf, n, _, _ in outs:
        _check(buf.cpu().numpy(), n)
