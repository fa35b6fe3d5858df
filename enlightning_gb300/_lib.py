"""ctypes binding of libenlightning_gpu.so (the product library).

The library is built in-tree by enlightning_gb300/build.py.  There is no CPU
fallback: if the shared object is missing or cannot be loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None

i32, i64, f64 = C.c_int, C.c_long, C.c_double
vp = C.c_void_p
ip = C.POINTER(C.c_int)
dp = C.POINTER(C.c_double)
REF_I = C.POINTER(C.c_int)
REF_D = C.POINTER(C.c_double)

# Symbols declared in include/enlightning_gpu.h, with their ctypes signature.
SIGNATURES = {
    "rhs_": (None, [REF_I] * 6 + [dp, dp, vp, vp, vp, vp, vp] + [REF_D] * 9 + [dp, REF_I, REF_D, REF_D, REF_I]),
    "runge_kutta_": (None, [REF_I] * 6 + [REF_D] * 4 + [vp, vp, vp, REF_I]),
    "update_state_": (None, [dp, dp] + [REF_I] * 6 + [vp, vp, vp] + [REF_D] * 11 + [REF_I]),
    "tag_cells_": (None, [REF_I] * 6 + [vp, vp, vp, REF_I, dp, REF_I]),
    "enl_set_stream": (i32, [vp]),
    "enl_get_last_error": (i32, []),
    "enl_error_string": (C.c_char_p, [i32]),
    "enl_set_rhs_variant": (i32, [i32]),
    "enl_get_rhs_variant": (i32, []),
    "enl_rhs": (i32, [i32] + [i32] * 6 + [dp, dp, vp, i64, i64, vp, vp, i64, i64, vp, vp]
                + [f64] * 7 + [dp, i32, f64, f64, vp]),
    "enl_phys_bc": (i32, [i32] * 6 + [ip, ip, i32, i32, vp, vp, vp, vp]),
    "enl_absorb": (i32, [i32] * 6 + [dp, dp, dp, dp, ip, f64, f64, f64, f64, vp, vp, vp]),
}


class EngineConfig(C.Structure):
    _fields_ = [
        ("nlevels", C.c_int), ("ratio", C.c_int), ("nx0", C.c_int), ("ny0", C.c_int),
        ("xlo", C.c_double * 2), ("dx0", C.c_double * 2), ("bc", C.c_int * 4),
        ("variant", C.c_int), ("precision", C.c_int), ("learned", C.c_int),
        ("weno_alpha", C.c_double), ("kappa", C.c_double), ("mu", C.c_double), ("muB", C.c_double),
        ("R", C.c_double), ("T_star_n", C.c_double), ("tau_n", C.c_double), ("c", C.c_double),
        ("c_lr", C.c_double), ("tol", C.c_double * 3), ("rho0", C.c_double), ("gamma1", C.c_double),
        ("c_p", C.c_double), ("p0", C.c_double), ("T0", C.c_double), ("c_v", C.c_double),
        ("absorb_width", C.c_double), ("rk_alpha1", C.c_double * 3), ("rk_alpha2", C.c_double * 3),
        ("rk_beta", C.c_double * 3), ("independent", C.c_int), ("dense", C.c_int),
        ("tile_order", C.c_int),
    ]


ENGINE_SIGNATURES = {
    "enl_engine_create": (C.c_int, [C.POINTER(EngineConfig), C.POINTER(C.c_void_p)]),
    "enl_engine_destroy": (C.c_int, [C.c_void_p]),
    "enl_engine_buffer": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_long),
                                    C.POINTER(C.c_long), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "enl_engine_set_patches": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "enl_engine_refine_init": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "enl_engine_fill": (C.c_int, [C.c_void_p, C.c_int]),
    "enl_engine_step": (C.c_int, [C.c_void_p, C.c_double]),
    "enl_engine_step_plain": (C.c_int, [C.c_void_p, C.c_double]),
    "enl_engine_graph_capture": (C.c_int, [C.c_void_p, C.c_double]),
    "enl_engine_graph_replay": (C.c_int, [C.c_void_p, C.c_int]),
    "enl_engine_tag": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "enl_engine_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "enl_engine_skipped_tiles": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                           C.POINTER(C.c_longlong)]),
    "enl_engine_health": (C.c_int, [C.c_void_p]),
    "enl_engine_launches_per_step": (C.c_int, [C.c_void_p, C.c_int]),
    "enl_engine_paint_source": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                          C.POINTER(C.c_double), C.c_double, C.c_double, C.c_int,
                                          C.POINTER(C.c_double), C.c_double]),
    "enl_engine_state_from_overpressure": (C.c_int, [C.c_void_p, C.c_int]),
    "enl_engine_set_adaptive_dt": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "enl_engine_packed_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "enl_engine_storage": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "enl_engine_graph_valid": (C.c_int, [C.c_void_p]),
    "enl_engine_set_level_order": (C.c_int, [C.c_void_p, C.c_int]),
    "enl_engine_set_schedule": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int]),
    "enl_engine_get_schedule": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int]),
    "enl_engine_autotune": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    "enl_engine_regrid": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]),
    "enl_engine_get_patches": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "enl_engine_regrid_timing": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "enl_engine_set_time": (C.c_int, [C.c_void_p, C.c_double, C.c_double]),
    "enl_engine_set_mics": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.c_int]),
    "enl_engine_mic_records": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]),
    "enl_cluster_tags": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                   C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "enl_cfl_dt_static": (C.c_int, [C.c_int] * 6 + [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_double,
                                                  C.c_double, C.c_void_p]),
    "enl_mlp_nparams": (C.c_int, []),
    "enl_mlp_forward": (C.c_int, [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]),
    "enl_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]),
    "enl_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float, C.c_float,
                               C.c_float, C.c_float, C.c_int]),
    "enl_engine_set_mlp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_float]),
    "enl_engine_harvest": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double), C.c_double, C.c_uint,
                                     C.c_void_p, C.c_void_p, C.c_long, C.c_void_p]),
    "enl_engine_profile": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_longlong)]),
    "enl_engine_profile_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                             C.POINTER(C.c_longlong)]),
    "enl_engine_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "enl_engine_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "enl_engine_download_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "enl_engine_upload_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "enl_engine_sync": (C.c_int, [C.c_void_p]),
    "enl_check_bounded_wait": (C.c_int, [C.c_int, C.c_int]),
    "enl_mlp_erf_error": (C.c_int, [C.POINTER(C.c_double)]),
    "enl_tile_neighbours": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                      C.POINTER(C.c_int)]),
    "enl_halo_segments": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                    C.POINTER(C.c_int)]),
    "enl_measure_fp_peaks": (C.c_int, [C.POINTER(C.c_double), C.c_int]),
    "enl_engine_time": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "enl_engine_tag_blocks": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]),
}
SIGNATURES.update(ENGINE_SIGNATURES)



class EnlightningError(RuntimeError):
    pass


def lib():
    """Load (building first if needed) the CUDA library; raises if unavailable."""
    global _lib
    if _lib is None:
        path = _build.build()
        if not os.path.exists(path):
            raise EnlightningError(f"CUDA library missing: {path}")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = lib().enl_error_string(status).decode()
        raise EnlightningError(f"{what}: {msg} (status {status})")


def check_sticky(what: str = "") -> None:
    check(lib().enl_get_last_error(), what)


def iref(v):
    return C.byref(C.c_int(int(v)))


def dref(v):
    return C.byref(C.c_double(float(v)))


def darr(values):
    a = (C.c_double * len(values))(*[float(x) for x in values])
    return a


def iarr(values):
    return (C.c_int * len(values))(*[int(x) for x in values])
