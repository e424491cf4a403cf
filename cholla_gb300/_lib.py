"""ctypes binding of libchollagb (include/cholla_gb300.h).

The library is the only compute path: if it is missing or cannot load, every call raises.
There is no host fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from .build import LIB, build

_lib = None

CGB_OK = 0
CGB_ERR_CUDA = 1
CGB_ERR_ARGS = 2
CGB_ERR_NOMEM = 3
CGB_ERR_NONFINITE = 4
CGB_ERR_TIMEOUT = 5
CGB_ERR_UNSUPPORTED = 6

CGB_STATUS_NEG_DENSITY = 1
CGB_STATUS_NONFINITE = 2
CGB_STATUS_TIMEOUT = 4
CGB_MAX_DIVB = 1.0e-9

PCM, PLMC, PPMC, PLMP, PPMP = 0, 1, 2, 3, 4
HLLC, ROE, HLLD, HLL, EXACT = 0, 1, 2, 3, 4
FP64, MIXED, FP64_FAST = 0, 1, 2


class CgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libchollagb error {code}: {msg}")
        self.code = code


class cgb_scheme(C.Structure):
    _fields_ = [
        ("reconstruction", C.c_int),
        ("riemann_solver", C.c_int),
        ("dual_energy", C.c_int),
        ("mhd", C.c_int),
        ("n_scalars", C.c_int),
        ("density_floor", C.c_int),
        ("temperature_floor", C.c_int),
        ("precision", C.c_int),
        ("gamma", C.c_double),
        ("U_floor", C.c_double),
    ]


_D = C.c_double
_I = C.c_int
_P = C.c_void_p

# name -> (restype, argtypes); every declaration of include/cholla_gb300.h
SIGNATURES = {
    "cgb_set_scheme": (_I, [C.POINTER(cgb_scheme)]),
    "cgb_get_scheme": (_I, [C.POINTER(cgb_scheme)]),
    "cgb_set_stream": (_I, [_P]),
    "cgb_last_error": (C.c_char_p, []),
    "cgb_version": (C.c_char_p, []),
    "cgb_vl_algorithm_3d": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _D, _P]),
    "cgb_vl_algorithm_3d_static": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _D,
                                        _P]),
    "cgb_vl_algorithm_1d": (_I, [_P, _I, _I, _I, _D, _D, _D, _I, _I]),
    "cgb_vl_algorithm_2d": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _I, _I]),
    "cgb_free_memory_vl_3d": (_I, []),
    "cgb_calc_dt_gpu": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, _D, C.POINTER(_D)]),
    "cgb_apply_temperature_floor": (_I, [_P, _I, _I, _I, _I, _I, _D]),
    "cgb_set_boundaries": (_I, [_P, _I, _I, _I, _I, _I, C.POINTER(_I)]),
    "cgb_max_magnetic_divergence": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, C.POINTER(_D)]),
    "cgb_check_magnetic_divergence": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, C.POINTER(_D)]),
    "cgb_check_status": (_I, [C.POINTER(_I)]),
    "cgb_debug_fail_alloc": (_I, [_I]),
    "cgb_box_create": (_I, [C.POINTER(_P), _I, _I, _I, _I, _D, _D, _D, C.POINTER(cgb_scheme), C.POINTER(_I)]),
    "cgb_box_destroy": (_I, [_P]),
    "cgb_box_n_fields": (_I, [_P]),
    "cgb_box_set_time": (_I, [_P, _D, _D]),
    "cgb_box_use_graph": (_I, [_P, _I]),
    "cgb_box_enable_timing": (_I, [_P, _I]),
    "cgb_box_kernel_times": (_I, [_P, C.POINTER(_D), C.POINTER(C.c_longlong)]),
    "cgb_box_advance": (_I, [_P, _P, _I, _D, _P]),
    "cgb_box_get_time": (_I, [_P, C.POINTER(_D), C.POINTER(_D)]),
    "cgb_box_check_status": (_I, [_P, C.POINTER(_I)]),
    "cgb_box_last_error": (C.c_char_p, []),
    "cgb_batch_create": (_I, [C.POINTER(_P), C.POINTER(cgb_scheme), _D, _P]),
    "cgb_batch_destroy": (_I, [_P]),
    "cgb_batch_job_bytes": (C.c_longlong, [_P, _I, _I, _I]),
    "cgb_batch_add": (_I, [_P, _P, _I, _I, _I, _I, _D, _D, _D, C.POINTER(_I), _D, C.POINTER(_I)]),
    "cgb_batch_remove": (_I, [_P, _I]),
    "cgb_batch_n_jobs": (_I, [_P]),
    "cgb_batch_set_chains": (_I, [_P, _I]),
    "cgb_batch_hold": (_I, [_P, _I, _I]),
    "cgb_selftest_conversions": (_I, [_P, C.c_longlong, _P, _P]),
    "cgb_selftest_fast_math": (_I, [_P, C.c_longlong, _P, _P]),
    "cgb_selftest_tma_timeout": (_I, [_P, C.c_uint, _P]),
    "cgb_set_tma": (_I, [_I]),
    "cgb_batch_set_solo_cells": (_I, [_P, C.c_longlong]),
    "cgb_batch_set_tiles": (_I, [_P, _I]),
    "cgb_selftest_fp64_rate": (_I, [_I, C.POINTER(C.c_double), _P]),
    "cgb_batch_step": (_I, [_P, _I]),
    "cgb_batch_job_time": (_I, [_P, _I, C.POINTER(_D), C.POINTER(_D)]),
    "cgb_batch_job_status": (_I, [_P, _I, C.POINTER(_I)]),
    "cgb_batch_last_error": (C.c_char_p, []),
    "cgb_ic_blast": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I, _P]),
    "cgb_ic_shock_tube": (_I, [_P, _I, _I, _I, _I, _I, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D,
                               _I, _P]),
}


def lib(auto_build: bool = True) -> C.CDLL:
    """Load libchollagb (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("CHOLLA_GB300_LIB", LIB))
    if not path.exists():
        if not auto_build:
            raise CgbError(CGB_ERR_ARGS, f"{path} not built")
        build()
    handle = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return handle


def check(rc: int) -> None:
    if rc != CGB_OK:
        msg = lib().cgb_last_error()
        raise CgbError(rc, msg.decode() if msg else "")
