"""The allocation-free point-mass entry point, through the C ABI.

ztm_gfm_pointmass_noalloc exists for callers that cannot allocate device
memory when they run a forward (a host that fixes its GPU memory up front,
work issued during stream capture, a real-time loop).  It keeps its scratch
in a fixed per-GPU array instead of a context workspace.  This test checks,
on two calls in a row (the second reusing the array the first left behind),
that it returns what the regular entry point returns, within the tolerance
of the point-mass tests (1e-12 normwise in double, 1e-5 in float), and that
a station count beyond the array is rejected.  It sits in a file of its own
that pytest collects last."""
import ctypes

import numpy as np
import pytest

import ztm_gb300
from helpers import rel_err, tfm_like_inputs

pytestmark = pytest.mark.gpu


def _noalloc(lib, grid, drho, surf, precision):
    import torch
    d = torch.tensor(drho, device="cuda")
    s = torch.tensor(surf, device="cuda")
    out = torch.full((grid.di * grid.dj,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.ztm_gfm_pointmass_noalloc(ctypes.byref(grid), ctypes.c_void_p(d.data_ptr()),
                                       ctypes.c_void_p(s.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), precision,
                                       ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = ztm_gb300.load()
    with ztm_gb300.GravityContext(0) as ctx:
        cases = [((31, 29, 17, 1, 2, 5), 21, ztm_gb300.PREC_FP64, 1e-12),
                 ((61, 61, 33, 1, 2, 10), 22, ztm_gb300.PREC_FP64, 1e-12),
                 ((61, 61, 33, 1, 2, 10), 23, ztm_gb300.PREC_FP32, 1e-5)]
        for dims, seed, prec, tol in cases:  # consecutive calls share the scratch
            g = ztm_gb300.make_grid(*dims)
            drho, surf = tfm_like_inputs(dims[0], dims[1], dims[2], dims[3], dims[4], seed=seed)
            rc, out = _noalloc(lib, g, drho, surf, prec)
            assert rc == ztm_gb300.OK
            ref = ctx.pointmass(g, drho, surf, precision="fp64" if prec == 0 else "fp32")
            assert np.all(np.isfinite(out))
            assert rel_err(out, ref) <= tol


def test_noalloc_rejects_more_stations_than_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = ztm_gb300.load()
    g = ztm_gb300.make_grid(800, 800, 2, 1, 1, 0)  # 640,000 interior stations
    d = torch.zeros(800 * 800 * 2, dtype=torch.float64, device="cuda")
    s = torch.zeros(800 * 800, dtype=torch.float64, device="cuda")
    out = torch.zeros(800 * 800, dtype=torch.float64, device="cuda")
    rc = lib.ztm_gfm_pointmass_noalloc(ctypes.byref(g), ctypes.c_void_p(d.data_ptr()),
                                       ctypes.c_void_p(s.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), 0, None)
    assert rc == ztm_gb300.ERR_RANGE
