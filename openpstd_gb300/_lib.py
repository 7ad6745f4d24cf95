"""ctypes binding of the in-tree CUDA library (include/pstd_gb300.h).

Loading fails loudly when ``libpstd_gb300.so`` has not been built: the
package has no CPU solver to fall back to.
"""
from __future__ import annotations

import ctypes
import os

from .config import c_config, c_domain_info

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpstd_gb300.so")

# status codes (include/pstd_gb300.h)
PSTD_OK = 0
PSTD_ERR_INVALID = 1
PSTD_ERR_NOT_CONFIGURED = 2
PSTD_ERR_CUDA = 3
PSTD_ERR_UNSUPPORTED = 4
PSTD_ERR_CALLBACK = 5
PSTD_ERR_NO_MEMORY = 6
PSTD_ERR_CANCELLED = 7
PSTD_ERR_TIMEOUT = 8
PSTD_ERR_IO = 9

FIELD = {"p0": 0, "px": 1, "py": 2, "vx": 3, "vy": 4}

WRITE_FRAME = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                               ctypes.POINTER(ctypes.c_float), ctypes.c_int64)
WRITE_SAMPLE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_float), ctypes.c_int64)
LOG = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p)
FRAME_BUFFER = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64)


class c_callbacks(ctypes.Structure):
    _fields_ = [("user", ctypes.c_void_p), ("write_frame", WRITE_FRAME), ("write_sample", WRITE_SAMPLE),
                ("log", LOG), ("frame_buffer", FRAME_BUFFER)]


# every symbol the header declares, with its signature
_P = ctypes.POINTER
_i32, _i64, _f32, _vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p
SIGNATURES = {
    "pstd_create": (ctypes.c_int, [_P(c_config), _P(c_callbacks), _P(_vp)]),
    "pstd_destroy": (None, [_vp]),
    "pstd_get_metadata": (ctypes.c_int, [_vp, _P(_i32), _P(_i32), _i32, _P(_i32)]),
    "pstd_run": (ctypes.c_int, [_vp, _P(c_callbacks)]),
    "pstd_run_sub": (ctypes.c_int, [_vp, _P(c_callbacks), _i32, _i32]),
    "pstd_advance": (ctypes.c_int, [_vp, _i32, _vp]),
    "pstd_reset": (ctypes.c_int, [_vp]),
    "pstd_synchronize": (ctypes.c_int, [_vp]),
    "pstd_steps_done": (ctypes.c_int, [_vp, _P(_i32)]),
    "pstd_get_receivers": (ctypes.c_int, [_vp, _i32, _i32, _P(_f32)]),
    "pstd_snapshot": (ctypes.c_int, [_vp, _i32, _i32, _P(_f32), _i64]),
    "pstd_create_batch": (ctypes.c_int, [_P(c_config), _i32, _P(c_callbacks), _P(_vp)]),
    "pstd_batch_scene": (ctypes.c_int, [_vp, _i32, _P(_i32)]),
    "pstd_batch_size": (ctypes.c_int, [_vp, _P(_i32), _P(_i32)]),
    "pstd_scene_build": (ctypes.c_int, [_P(c_config), _P(_vp)]),
    "pstd_scene_strip_runs": (ctypes.c_int, [_vp, _i32, _i32, _P(_i32), _i32, _P(_i32)]),
    "pstd_scene_domain_count": (ctypes.c_int, [_vp, _P(_i32)]),
    "pstd_scene_domain_info": (ctypes.c_int, [_vp, _i32, _P(c_domain_info)]),
    "pstd_scene_neighbours": (ctypes.c_int, [_vp, _i32, _i32, _P(_i32), _i32, _P(_i32)]),
    "pstd_scene_attenuation": (ctypes.c_int, [_vp, _i32, _P(_f32), _P(_f32), _P(_f32), _P(_f32)]),
    "pstd_profile_passes": (ctypes.c_int, [_vp, _i32, _vp, _P(_f32), _P(_f32), _P(_i32), _P(_i32)]),
    "pstd_plan_info": (ctypes.c_int, [_vp, ctypes.c_char_p, _i32]),
    "pstd_work_counts": (ctypes.c_int, [_vp, _P(_i64), _P(_i64), _P(_i32)]),
    "pstd_server_create": (ctypes.c_int, [_i64, _i32, _P(c_callbacks), _P(_vp)]),
    "pstd_server_destroy": (None, [_vp]),
    "pstd_server_submit": (ctypes.c_int, [_vp, _P(c_config), _i32, _i32, _P(_i64)]),
    "pstd_server_tick": (ctypes.c_int, [_vp, _i32, _P(_i32)]),
    "pstd_server_poll": (ctypes.c_int, [_vp, _i64, _P(_i32), _P(_i32), _P(_i64)]),
    "pstd_server_result": (ctypes.c_int, [_vp, _i64, _P(_f32), _i64, _P(_f32), _i64]),
    "pstd_server_cancel": (ctypes.c_int, [_vp, _i64]),
    "pstd_stage_variants": (ctypes.c_int, [_i32, ctypes.c_char_p, _i32, _P(_i32)]),
    "pstd_transform_gain": (ctypes.c_int, [_i32, _P(_i32), _i32, _i32, _i32, _P(ctypes.c_double)]),
    "pstd_host_register": (ctypes.c_int, [_vp, _i64]),
    "pstd_host_unregister": (ctypes.c_int, [_vp]),
    "pstd_server_stats": (ctypes.c_int, [_vp, _P(_i64)]),
    "pstd_server_launch_stats": (ctypes.c_int, [_vp, _P(_i64)]),
    "pstd_solve_noalloc": (ctypes.c_int, [_P(c_config), _i32, _vp, _i64, _vp, _i64, _vp]),
    "pstd_spectral_plan": (ctypes.c_int, [_P(c_config), _vp, _vp, _vp, _vp, _P(_i64)]),
    "pstd_file_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _i32, _P(_vp)]),
    "pstd_file_close": (None, [_vp]),
    "pstd_file_get_scene": (ctypes.c_int, [_vp, _i32, _P(c_config)]),
    "pstd_file_set_scene": (ctypes.c_int, [_vp, _i32, _P(c_config)]),
    "pstd_file_initialize_results": (ctypes.c_int, [_vp]),
    "pstd_file_delete_results": (ctypes.c_int, [_vp]),
    "pstd_file_save_frame": (ctypes.c_int, [_vp, _i32, _P(_f32), _i64]),
    "pstd_file_frame_count": (ctypes.c_int, [_vp, _i32, _P(_i32)]),
    "pstd_file_get_frame": (ctypes.c_int, [_vp, _i32, _i32, _P(_f32), _i64, _P(_i64)]),
    "pstd_file_append_samples": (ctypes.c_int, [_vp, _i32, _P(_f32), _i64]),
    "pstd_file_get_samples": (ctypes.c_int, [_vp, _i32, _P(_f32), _i64, _P(_i64)]),
    "pstd_file_commit": (ctypes.c_int, [_vp]),
    "pstd_file_rollback": (ctypes.c_int, [_vp]),
    "pstd_file_last_error": (ctypes.c_char_p, []),
    "pstd_archive_encode": (ctypes.c_int, [_P(c_config), ctypes.c_char_p, _i64, _P(_i64)]),
    "pstd_last_error": (ctypes.c_char_p, []),
    "pstd_version": (ctypes.c_char_p, []),
}

_lib = None


class PSTDError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[pstd status {code}] {message}")
        self.code = code


def lib():
    """Load libpstd_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m openpstd_gb300.build` "
                               "(the package has no CPU solver)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != PSTD_OK:
        raise PSTDError(rc, lib().pstd_last_error().decode())
