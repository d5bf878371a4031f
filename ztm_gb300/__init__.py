"""ztm_gb300: GB300-native gravity forward model and adjoint behind ZTM's
gravity call surface (TFM.cpp:83-99, GFM_GPU.cu).  The compute path is
libztmgrav.so (hand-written sm_103a CUDA behind the C ABI of
include/ztm_grav.h); this package is its Python binding."""
from ._lib import (ERR_ALLOC, ERR_ARG, ERR_CUDA, ERR_NODEV, ERR_RANGE, ERR_TIMEOUT, EXPORTS,
                   FLAG_DEVICE_PTRS, OK, PREC_FP32, PREC_FP64, PREC_MIXED, load, lib_path)
from .gfm import (DEFAULT_G, GravityContext, GravityError, make_grid, make_imesh, make_mesh)

__all__ = [
    "GravityContext", "GravityError", "make_grid", "make_mesh", "make_imesh", "load", "lib_path",
    "EXPORTS", "DEFAULT_G", "PREC_FP64", "PREC_FP32", "PREC_MIXED", "FLAG_DEVICE_PTRS", "OK",
    "ERR_ARG", "ERR_ALLOC", "ERR_CUDA", "ERR_TIMEOUT", "ERR_NODEV", "ERR_RANGE",
]
