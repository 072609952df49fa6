"""ctypes bindings of libgraspgpu (the C ABI in include/grasp_gpu.h).

The library is built in-tree (grasp_gb300/_build). Loading fails loudly
when it is missing: there is no CPU fallback for the GPU path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_i64 = C.POINTER(C.c_int64)
_int = C.POINTER(C.c_int)
_u8 = C.POINTER(C.c_uint8)

_gpu = None


class GGList(C.Structure):
    _fields_ = [("nlab", C.c_int64), ("lab", _i32), ("start", _i64), ("loc", _i32), ("coeff", _d)]


class GGCof(C.Structure):
    """gg_cof: one orbital's SETCOF lists (include/grasp_gpu.h)."""
    _fields_ = [("ny", C.c_int), ("nya", C.POINTER(C.c_int32)), ("ya", C.POINTER(C.c_double)),
                ("nx", C.c_int), ("nxa", C.POINTER(C.c_int32)), ("xa", C.POINTER(C.c_double)),
                ("nd", C.c_int), ("nda", C.POINTER(C.c_int32)), ("da", C.POINTER(C.c_double))]


class GGDvdParams(C.Structure):
    _fields_ = [
        ("flavour", C.c_int), ("precision", C.c_int), ("lim", C.c_int), ("maxiter", C.c_int),
        ("critr", C.c_double), ("critc", C.c_double), ("crite", C.c_double), ("robust", C.c_int),
        ("mblock", C.c_int), ("nstart", C.c_int), ("start", _d),
    ]


# symbol name -> (restype, argtypes); every symbol include/grasp_gpu.h declares
GPU_SYMBOLS = {
    "gg_last_error": (C.c_char_p, []),
    "gg_version": (C.c_int, []),
    "gg_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gg_ctx_destroy": (C.c_int, [C.c_void_p]),
    "gg_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "gg_release_memory": (C.c_int, [C.c_int]),
    "gg_set_grid": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, _d, _d, _d, _d]),
    "gg_get_grid": (C.c_int, [C.c_void_p, _d, _d, _d]),
    "gg_set_orbitals": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _int, _int, _d, _d]),
    "gg_genintrk": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _i64, _int]),
    "gg_get_rk_table": (C.c_int, [C.c_void_p, _i32, _d, _i32]),
    "gg_rkintc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _d]),
    "gg_slater": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _d]),
    "gg_ypot": (C.c_int, [C.c_void_p, C.c_int, _i32, _d, _d]),
    "gg_xpot": (C.c_int, [C.c_void_p, C.c_int, _i32, _d, _d, _d]),
    "gg_cofpot": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(GGCof), C.c_int, _i32, _d, C.c_double, _d,
                            _d, _d]),
    "gg_setlag": (C.c_int, [C.c_void_p, C.c_int, _i32, _d, _int, C.POINTER(GGCof), _d]),
    "gg_genintbreit": (C.c_int, [C.c_void_p, C.c_int, C.c_double, _d, C.c_double, _i64, _int]),
    "gg_setcof_prepare": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), _int, C.POINTER(_d),
                                    C.POINTER(_d), C.c_int]),
    "gg_setcof": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, _int, _i32, _d, _int, _i32, _d, _int, _i32,
                            _d]),
    "gg_get_breit_table": (C.c_int, [C.c_void_p, C.c_int, _i32, _d, _i32]),
    "gg_brint": (C.c_int, [C.c_void_p] + [C.c_int] * 6 + [_d]),
    "gg_brintf": (C.c_int, [C.c_void_p, C.c_int, _i32, C.c_double, _d, C.c_double, _d]),
    "gg_slater_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _d]),
    "gg_rinti": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _d]),
    "gg_iabint_table": (C.c_int, [C.c_void_p, _d]),
    "gg_hmat_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, _i64, _i32, C.POINTER(C.c_void_p)]),
    "gg_hmat_destroy": (C.c_int, [C.c_void_p]),
    "gg_hmat_create_view": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "gg_setham_upload": (C.c_int, [C.c_void_p, C.c_void_p, _u8, C.POINTER(GGList), C.c_int, C.POINTER(GGList)]),
    "gg_setham_assemble": (C.c_int, [C.c_void_p, C.c_void_p, _d]),
    "gg_setham": (C.c_int, [C.c_void_p, C.c_void_p, _u8, C.POINTER(GGList), C.c_int, C.POINTER(GGList), _d]),
    "gg_hmat_get_emt": (C.c_int, [C.c_void_p, _d]),
    "gg_hmat_set_emt": (C.c_int, [C.c_void_p, _d]),
    "gg_spicmv2": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, _d, _d, C.c_int]),
    "gg_hmat_create_host": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, _i64, _i32, _d, C.c_double, C.c_int,
                                      C.POINTER(C.c_void_p)]),
    "gg_hmat_host_precision": (C.c_int, [C.c_void_p]),
    "gg_spodmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, _d, _d]),
    "gg_hmat_create_packed": (C.c_int, [C.c_void_p, C.c_int, _d, C.POINTER(C.c_void_p)]),
    "gg_host_read_timing": (C.c_int, [C.c_void_p, C.c_size_t, C.c_int, C.c_int, _d]),
    "gg_maneig": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(GGDvdParams), _d, _d, _int, _int, _int]),
    "gg_maneig_batched": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), _int, C.POINTER(GGDvdParams), _d,
                                    _d, _int, _int, _int]),
    "gg_stage_stat": (C.c_double, [C.c_void_p, C.c_int]),
    "gg_launch_count": (C.c_longlong, []),
    "gg_alloc_count": (C.c_longlong, []),
    "gg_test_stall_rk_tile": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_host_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "gg_host_unregister": (C.c_int, [C.c_void_p]),
    "gg_event_record": (C.c_int, [C.c_void_p, C.c_int]),
    "gg_event_elapsed": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _d]),
    "gg_matvec_timing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, _d, _d]),
    "gg_spmm_timing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, _d, _d]),
    "gg_projected_eig": (C.c_int, [C.c_int, _d, C.c_int, C.c_int, _d, _d]),
    "gg_hmat_tune": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _int, _int, _d]),
    "gg_hmat_tune_force": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "gg_batched_tune_info": (C.c_int, [C.c_void_p, _int, _int, _d]),
    "gg_tune_variant_name": (C.c_char_p, [C.c_int, C.c_int]),
}


def _bind(lib, table):
    for name, (res, args) in table.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def lib_path():
    return _build.LIB_GPU


def ensure_built():
    if not os.path.exists(_build.LIB_GPU):
        _build.build()


def gpu():
    """libgraspgpu, loaded on first use. Raises if it is missing."""
    global _gpu
    if _gpu is None:
        if not os.path.exists(_build.LIB_GPU):
            raise RuntimeError(
                f"libgraspgpu.so not found at {_build.LIB_GPU}: build it with `python -m grasp_gb300.build` "
                "(there is no CPU fallback)")
        _gpu = _bind(C.CDLL(_build.LIB_GPU), GPU_SYMBOLS)
    return _gpu


class GGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def check(status):
    if status != 0:
        msg = gpu().gg_last_error()
        raise GGError(status, msg.decode() if msg else "")
    return status


def ptr(a, t):
    return a.ctypes.data_as(t)
