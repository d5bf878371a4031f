"""C ABI checks that need no GPU: the library loads, exports every symbol
that include/ztm_grav.h declares, and fails cleanly without a device."""
import ctypes
import os
import re

import pytest

import ztm_gb300
from ztm_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ztm_grav.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ztm_[a-z_0-9]+)\s*\(", txt)))


def test_header_symbols_listed():
    assert set(header_symbols()) == set(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = ztm_gb300.load()
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_version():
    assert ztm_gb300.load().ztm_version() >= 100


def test_null_and_bad_arguments_do_not_crash():
    lib = ztm_gb300.load()
    assert lib.ztm_ctx_create(0, None) == _lib.ERR_ARG
    assert lib.ztm_last_error(None) == b"null context"
    assert lib.ztm_gfm_prism(None, None, None, 0, None, None, None) == _lib.ERR_ARG
    assert lib.ztm_ctx_sync(None) == _lib.ERR_ARG
    assert lib.ztm_gfm_pointmass_model(None, None, None, None, None, None, None, None, 0,
                                       0) == _lib.ERR_ARG
    assert lib.ztm_gfm_pointmass_adjoint(None, None, None, None, 0, None, None, None, 0,
                                         0) == _lib.ERR_ARG
    assert lib.ztm_gfm_pointmass_misfit(None, None, None, None, 0, None, None, 0.0, 1.0, None,
                                        None, None, None, None, 0, 0) == _lib.ERR_ARG
    assert lib.ztm_gfm_pointmass_model_misfit(None, None, None, None, None, None, None, None, 0.0,
                                              1.0, None, None, None, None, None, None, 0,
                                              0) == _lib.ERR_ARG
    assert lib.ztm_lm_steps(None, None, 0, 0, None, None, None, None, 0, None, None,
                            0) == _lib.ERR_ARG
    assert lib.ztm_ctx_tuning(None, None, 0) == _lib.ERR_ARG
    lib.ztm_ctx_destroy(None)


def test_context_without_device_reports_nodev():
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a device is present")
    h = ctypes.c_void_p()
    rc = ztm_gb300.load().ztm_ctx_create(0, ctypes.byref(h))
    assert rc == _lib.ERR_NODEV
    with pytest.raises(ztm_gb300.GravityError):
        ztm_gb300.GravityContext(0)
