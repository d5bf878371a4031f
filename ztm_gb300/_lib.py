"""ctypes binding of include/ztm_grav.h (libztmgrav.so).

This is the same binding a Python caller of the C ABI would write; the
reference-side C++ binding is the header itself.  The library is built
in-tree by ztm_gb300._build; there is no fallback: if the shared library is
missing, every call raises."""
import ctypes
import os

from . import _build

# status codes
OK = 0
ERR_ARG = -1
ERR_ALLOC = -2
ERR_CUDA = -3
ERR_TIMEOUT = -4
ERR_NODEV = -5
ERR_RANGE = -6

PREC_FP64 = 0
PREC_FP32 = 1
PREC_MIXED = 2
FLAG_DEVICE_PTRS = 1

# every symbol include/ztm_grav.h declares
EXPORTS = (
    "ztm_version", "ztm_ctx_create", "ztm_ctx_destroy", "ztm_last_error",
    "ztm_ctx_set_stream", "ztm_ctx_stream", "ztm_ctx_launches", "ztm_ctx_sync",
    "ztm_gfm_pointmass", "ztm_gfm_prism", "ztm_gfm_prism_list", "ztm_gfm_adjoint",
    "ztm_gfm_interface", "ztm_gfm_interface_adjoint", "ztm_gfm_interface_misfit",
    "ztm_gfm_batch", "ztm_ctx_profile", "ztm_ctx_profile_read", "ztm_measure_peak",
    "ztm_invert_interface", "ztm_gfm_pointmass_noalloc", "ztm_density_build",
    "ztm_gfm_pointmass_model", "ztm_gfm_interface_jvp", "ztm_gfm_pointmass_adjoint",
    "ztm_gfm_pointmass_misfit", "ztm_gfm_pointmass_model_misfit", "ztm_ctx_count_forms",
    "ztm_ctx_form_counts", "ztm_ctx_test_timeout", "ztm_invert_interface_gn",
    "ztm_lm_steps", "ztm_ctx_tuning",
)


class Grid(ctypes.Structure):
    _fields_ = [("di", ctypes.c_int), ("dj", ctypes.c_int), ("dk", ctypes.c_int),
                ("fh", ctypes.c_int), ("fv", ctypes.c_int), ("bfr", ctypes.c_int),
                ("threshold", ctypes.c_double), ("scale", ctypes.c_double)]


class Mesh(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("z_top", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)]


class IMesh(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("z_base", ctypes.c_double)]


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("flags", ctypes.c_int),
                ("G", ctypes.c_double), ("near_q", ctypes.c_double),
                ("tile", ctypes.c_int), ("chunk", ctypes.c_int)]


class DensityParams(ctypes.Structure):
    _fields_ = [("di", ctypes.c_int), ("dj", ctypes.c_int), ("dk", ctypes.c_int),
                ("fh", ctypes.c_int), ("fv", ctypes.c_int), ("vm", ctypes.c_double),
                ("ro", ctypes.c_double), ("dr", ctypes.c_double), ("rc", ctypes.c_double * 10)]


class Job(ctypes.Structure):
    _fields_ = [("mesh", Mesh), ("nmodels", ctypes.c_int),
                ("rho", ctypes.c_void_p), ("ns", ctypes.c_int),
                ("sxyz", ctypes.c_void_p), ("gz", ctypes.c_void_p)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SIGS = {
    "ztm_version": (_I, []),
    "ztm_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "ztm_ctx_destroy": (None, [_P]),
    "ztm_last_error": (ctypes.c_char_p, [_P]),
    "ztm_ctx_set_stream": (_I, [_P, _P]),
    "ztm_ctx_stream": (_P, [_P]),
    "ztm_ctx_launches": (_LL, [_P]),
    "ztm_ctx_sync": (_I, [_P]),
    "ztm_gfm_pointmass": (_I, [_P, ctypes.POINTER(Grid), _P, _P, _LL, _P, _P, _I, _I]),
    "ztm_gfm_pointmass_noalloc": (_I, [ctypes.POINTER(Grid), _P, _P, _P, _I, _P]),
    "ztm_gfm_prism": (_I, [_P, ctypes.POINTER(Mesh), _P, _I, _P, _P, ctypes.POINTER(Opts)]),
    "ztm_gfm_prism_list": (_I, [_P, _LL, _P, _P, _I, _P, _P, ctypes.POINTER(Opts)]),
    "ztm_gfm_adjoint": (_I, [_P, ctypes.POINTER(Mesh), _I, _P, _P, _P, ctypes.POINTER(Opts)]),
    "ztm_gfm_interface": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _I, _P, _P,
                               ctypes.POINTER(Opts)]),
    "ztm_gfm_interface_adjoint": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _I, _P, _P, _P, _P,
                                       ctypes.POINTER(Opts)]),
    "ztm_gfm_interface_jvp": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _P, _I, _P, _P,
                                   ctypes.POINTER(Opts)]),
    "ztm_gfm_interface_misfit": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _I, _P, _P, _P, _P,
                                      _P, _P, ctypes.POINTER(Opts)]),
    "ztm_gfm_batch": (_I, [_P, ctypes.POINTER(Job), _I, ctypes.POINTER(Opts)]),
    "ztm_density_build": (_I, [_P, ctypes.POINTER(DensityParams), _P, _P, _P, _P,
                               ctypes.POINTER(_LL), _I]),
    "ztm_gfm_pointmass_model": (_I, [_P, ctypes.POINTER(DensityParams), ctypes.POINTER(Grid),
                                     _P, _P, _P, _P, _P, _I, _I]),
    "ztm_gfm_pointmass_adjoint": (_I, [_P, ctypes.POINTER(Grid), _P, _P, _LL, _P, _P, _P, _I, _I]),
    "ztm_gfm_pointmass_misfit": (_I, [_P, ctypes.POINTER(Grid), _P, _P, _LL, _P, _P,
                                      ctypes.c_double, ctypes.c_double, _P, _P, _P, _P, _P, _I,
                                      _I]),
    "ztm_gfm_pointmass_model_misfit": (_I, [_P, ctypes.POINTER(DensityParams),
                                            ctypes.POINTER(Grid), _P, _P, _P, _P, _P,
                                            ctypes.c_double, ctypes.c_double, _P, _P, _P, _P, _P,
                                            _P, _I, _I]),
    "ztm_invert_interface_gn": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _I, _P, _P, ctypes.c_double,
                                     _I, _I, ctypes.POINTER(Opts), _P, ctypes.POINTER(_I)]),
    "ztm_lm_steps": (_I, [_P, _P, _I, _I, _P, _P, _P, _P, _I, _P, _P, _I]),
    "ztm_ctx_tuning": (_I, [_P, ctypes.POINTER(_I), _I]),
    "ztm_ctx_count_forms": (_I, [_P, _I]),
    "ztm_ctx_form_counts": (_I, [_P, ctypes.POINTER(_LL)]),
    "ztm_ctx_test_timeout": (_I, [_P, ctypes.c_uint]),
    "ztm_ctx_profile": (_I, [_P, _I]),
    "ztm_ctx_profile_read": (_I, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(_LL)]),
    "ztm_measure_peak": (_I, [_P, _I, ctypes.POINTER(ctypes.c_double)]),
    "ztm_invert_interface": (_I, [_P, ctypes.POINTER(IMesh), _P, _P, _I, _P, _P, ctypes.c_double, _I,
                                  ctypes.POINTER(Opts), _P, ctypes.POINTER(_I)]),
}

_lib = None


def lib_path():
    return _build.LIB


def load():
    """Load libztmgrav.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError("libztmgrav.so is not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
