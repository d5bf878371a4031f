"""The GFM drop-in executable keeps the /dev/shm file contract of
TFM.cpp:90-94 / GFM_GPU.cu:24-34 (here redirected to a temp dir)."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import ztm_gb300
from ztm_gb300 import _build
from helpers import rel_err, tfm_like_inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_shim(tmp, dims, env_extra=None):
    env = dict(os.environ, ZTM_GFM_DIR=str(tmp), ZTM_GFM_DIMS=",".join(map(str, dims)))
    env.update(env_extra or {})
    return subprocess.run([_build.SHIM], env=env, capture_output=True, text=True, timeout=120)


def write_inputs(tmp, dims, seed=0):
    di, dj, dk, fh, fv, bfr = dims
    drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=seed)
    drho.astype(np.float32).tofile(os.path.join(tmp, "R.dat"))
    surf.astype(np.float32).tofile(os.path.join(tmp, "S.dat"))
    return drho, surf


def test_cpp_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "ztm_grav.hpp"\nint main(){std::vector<double> a,b,c; std::vector<int> n;'
                   ' return ztm::gfm(a,b,c,n,3,3,3) == 0;}\n')
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_shim_missing_files(tmp_path):
    assert os.path.exists(_build.SHIM)
    r = run_shim(tmp_path, (11, 11, 5, 1, 2, 2))
    assert r.returncode == 1


def test_shim_without_device_reports_library_error(tmp_path):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a device is present")
    write_inputs(tmp_path, (11, 11, 5, 1, 2, 2))
    assert run_shim(tmp_path, (11, 11, 5, 1, 2, 2)).returncode == 2


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_shim_file_protocol(tmp_path, prec):
    dims = (31, 29, 17, 1, 2, 5)
    drho, surf = write_inputs(tmp_path, dims, seed=2)
    r = run_shim(tmp_path, dims, {"ZTM_GFM_PRECISION": prec})
    assert r.returncode == 0, r.stderr
    g = np.fromfile(os.path.join(tmp_path, "G.dat"), dtype=np.float32)
    grid = ztm_gb300.make_grid(*dims)
    ref = oracle.pointmass_tfm(grid, drho.astype(np.float32).astype(np.float64),
                               surf.astype(np.float32).astype(np.float64))
    assert g.size == 31 * 29
    assert rel_err(g, ref) <= 1e-5


@pytest.mark.gpu
def test_shim_reference_default_dims_short_input(tmp_path):
    """Default dims 61,61,35 read 61*61*69 values while TFM writes
    61*61*65 (dk=33): the tail is zero-filled."""
    dims_tfm = (61, 61, 33, 1, 2, 10)
    drho, surf = write_inputs(tmp_path, dims_tfm, seed=3)
    env = dict(os.environ, ZTM_GFM_DIR=str(tmp_path))
    env.pop("ZTM_GFM_DIMS", None)
    r = subprocess.run([_build.SHIM], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    g = np.fromfile(os.path.join(tmp_path, "G.dat"), dtype=np.float32)
    ref = oracle.pointmass_tfm(ztm_gb300.make_grid(*dims_tfm),
                               drho.astype(np.float32).astype(np.float64),
                               surf.astype(np.float32).astype(np.float64))
    assert rel_err(g, ref) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_shim_threshold_is_gf_float_rule(tmp_path, prec):
    """GF selects fabs(rho) > .001f on the float values of R.dat
    (GFM_GPU.cu:19): nodes stored as exactly 0.001f (whose double value is
    just above 0.001) and -0.001f contribute nothing, in either precision."""
    dims = (21, 19, 9, 1, 2, 3)
    drho, surf = tfm_like_inputs(*dims[:3], seed=4)
    r32 = drho.astype(np.float32)
    at = np.nonzero(r32 != 0)[0][::7]
    r32[at[::2]] = np.float32(0.001)
    r32[at[1::2]] = np.float32(-0.001)
    r32.tofile(os.path.join(tmp_path, "R.dat"))
    surf.astype(np.float32).tofile(os.path.join(tmp_path, "S.dat"))
    r = run_shim(tmp_path, dims, {"ZTM_GFM_PRECISION": prec})
    assert r.returncode == 0, r.stderr
    g = np.fromfile(os.path.join(tmp_path, "G.dat"), dtype=np.float32)
    grid = ztm_gb300.make_grid(*dims)
    r64 = r32.astype(np.float64)
    nn = np.nonzero(np.abs(r32) > np.float32(0.001))[0]
    ref = oracle.pointmass_tfm(grid, r64, surf.astype(np.float32).astype(np.float64), nn=nn)
    assert rel_err(g, ref) <= 1e-5
    # the double threshold would have counted the 0.001f nodes (6e-3 here)
    wrong = oracle.pointmass_tfm(grid, r64, surf.astype(np.float32).astype(np.float64))
    assert rel_err(wrong, ref) > 1e-3
