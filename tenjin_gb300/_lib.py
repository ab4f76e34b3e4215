"""ctypes binding of libtenjin_gpu.so (include/tenjin_gpu.h).

The library is the product: there is no CPU fallback. Loading fails loudly
if the shared object has not been built (tenjin_gb300.build.build()).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

TJ_MAX_MATERIALS = 4
TJ_MAX_EOS_PARAMS = 16

TJ_OK = 0
ERRORS = {
    -1: "TJ_ERR_ARG", -2: "TJ_ERR_CUDA", -3: "TJ_ERR_NAN", -4: "TJ_ERR_WAVESPEED",
    -5: "TJ_ERR_ALPHA", -6: "TJ_ERR_PLASTIC", -7: "TJ_ERR_STATE", -8: "TJ_ERR_ROOT",
}
TJ_PRECISION_FP64 = 0
TJ_PRECISION_MIXED = 1
TJ_PRECISION_FUSED64 = 2


class TjMaterial(ctypes.Structure):
    _fields_ = [("phase", ctypes.c_int), ("eos", ctypes.c_int), ("nparams", ctypes.c_int),
                ("params", ctypes.c_double * TJ_MAX_EOS_PARAMS), ("yield_stress", ctypes.c_double)]


class TjParams(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("n_materials", ctypes.c_int), ("n_mixtures", ctypes.c_int),
                ("SOLID", ctypes.c_int), ("THINC", ctypes.c_int), ("RADIAL", ctypes.c_int),
                ("PLASTIC", ctypes.c_int), ("REACTIVE", ctypes.c_int), ("MUSCL", ctypes.c_int),
                ("nghost", ctypes.c_int), ("lo_bc", ctypes.c_int * 3), ("hi_bc", ctypes.c_int * 3),
                ("CFL", ctypes.c_double), ("THINCbeta", ctypes.c_double), ("precision", ctypes.c_int),
                ("materials", TjMaterial * TJ_MAX_MATERIALS)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_PD = ctypes.POINTER(ctypes.c_double)
_PI = ctypes.POINTER(ctypes.c_int)

# (name, restype, argtypes) for every entry point of include/tenjin_gpu.h
SIGNATURES = [
    ("tj_create", _I, [ctypes.POINTER(TjParams), ctypes.POINTER(_P)]),
    ("tj_destroy", _I, [_P]),
    ("tj_last_error", _I, [_P, ctypes.c_char_p, ctypes.c_ulong]),
    ("tj_ncomp", _I, [_P]),
    ("tj_set_domains", _I, [_P, _I, _PI, _PD]),
    ("tj_set_boxes", _I, [_P, _I, _I, _PI]),
    ("tj_set_max_grid_size", _I, [_P, _I, _I]),
    ("tj_num_boxes", _I, [_P, _I]),
    ("tj_get_box", _I, [_P, _I, _I, _PI]),
    ("tj_num_cells", _I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("tj_upload_state", _I, [_P, _I, _I, _PD, _I, _I]),
    ("tj_download_state", _I, [_P, _I, _I, _PD, _I, _I]),
    ("tj_upload_domain", _I, [_P, _I, _PD]),
    ("tj_download_domain", _I, [_P, _I, _PD]),
    ("tj_set_primitive", _I, [_P, _I, _PD]),
    ("tj_compute_dt", _I, [_P, _PD]),
    ("tj_advance", _I, [_P, _D]),
    ("tj_advance_stage", _I, [_P, _I, _D]),
    ("tj_plastic_update", _I, [_P, _D]),
    ("tj_reactive_update", _I, [_P, _D]),
    ("tj_geometric_source", _I, [_P, _D]),
    ("tj_cleanup_v", _I, [_P]),
    ("tj_cleanup_alpha", _I, [_P]),
    ("tj_cons_to_prim", _I, [_P]),
    ("tj_prim_to_cons", _I, [_P]),
    ("tj_contains_nan", _I, [_P, _PI]),
    ("tj_conservation_sums", _I, [_P, _PD]),
    ("tj_download_component", _I, [_P, _I, _I, _PD]),
    ("tj_step", _I, [_P, _D]),
    ("tj_run", _I, [_P, _I, _D, _PI, _PD]),
    ("tj_get_time", _I, [_P, _PD, _PI, _PD]),
    ("tj_set_time", _I, [_P, _D, _I]),
    ("tj_status", _I, [_P]),
    ("tj_synchronize", _I, [_P]),
    ("tj_launch_count", _I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("tj_get_stream", _I, [_P, ctypes.POINTER(_P)]),
    ("tj_set_profiling", _I, [_P, _I]),
    ("tj_kernel_time", _I, [_P, ctypes.c_char_p, _PD, ctypes.POINTER(ctypes.c_longlong)]),
    ("tj_compute_dt_noalloc", _I, [ctypes.POINTER(TjParams), _PI, _PD, ctypes.c_void_p, _PD, ctypes.c_void_p]),
    ("tj_kernel_config", _I, [_P, ctypes.c_char_p, ctypes.c_ulong]),
    ("tj_forward", _I, [_P, _I, ctypes.c_void_p, _PD, _I, _PD, _I]),
    ("tj_backward", _I, [_P, _I, ctypes.c_void_p, ctypes.c_void_p, _PD]),
    ("tj_tangent", _I, [_P, _I, ctypes.c_void_p, ctypes.c_void_p, _PD, _PD, _I, _PD, ctypes.c_void_p,
                        ctypes.c_void_p]),
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load():
    """Load the library (build it first if the sources are newer)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run tenjin_gb300.build.build() (no CPU fallback exists)")
        L = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class TjError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
