"""ctypes binding of libsarbp.so (the C ABI declared in include/sarbp.h).

There is no fallback: if the library cannot be loaded, every focusing call
raises.  ``load()`` builds the library first when it is missing or stale.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

SARBP_OK = 0
SARBP_EINVAL = -1
SARBP_EWORKSPACE = -2
SARBP_ECUDA = -3
SARBP_ETIMEOUT = -4
SARBP_ERANGE = -5
SARBP_EDEVICE = -6
SARBP_ECANCELED = -7

CTR_AMBIGUOUS = 0
CTR_WINDOW_MISS = 1
CTR_CHUNKS = 2
CTR_TIMEOUTS = 3
NUM_COUNTERS = 8
PREVIEW_SCRATCH_BYTES = 16384


class SarbpError(RuntimeError):
    """A libsarbp call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"libsarbp status {status}: {message}")
        self.status = status


class Scene(C.Structure):
    """struct sarbp_scene (include/sarbp.h)."""

    _fields_ = [
        ("dim0", C.c_int64), ("dim1", C.c_int64),
        ("dem_x", C.c_void_p), ("dem_y", C.c_void_p), ("dem_z", C.c_void_p),
        ("mask", C.c_void_p), ("index", C.c_void_p), ("sint", C.c_void_p),
        ("traj_x", C.c_void_p), ("traj_y", C.c_void_p), ("traj_z", C.c_void_p),
        ("raw", C.c_void_p),
        ("nra", C.c_int64), ("naz", C.c_int64), ("raw_pitch", C.c_int64),
        ("near_range", C.c_double), ("delta_range", C.c_double), ("lambda_", C.c_double),
    ]


class Tuning(C.Structure):
    """struct sarbp_tuning (include/sarbp.h)."""

    _fields_ = [
        ("chunk", C.c_int32), ("tile0", C.c_int32), ("tile1", C.c_int32),
        ("staged", C.c_int32), ("window", C.c_int32), ("stage", C.c_int32),
        ("wait_polls", C.c_int32), ("withhold", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {"chunk": self.chunk, "tile0": self.tile0, "tile1": self.tile1,
                "staged": self.staged, "window": self.window, "stage": self.stage}


_P = C.c_void_p
# name -> (restype, argtypes); every symbol include/sarbp.h declares.
SIGNATURES = {
    "sarbp_version": (C.c_int, []),
    "sarbp_last_error": (C.c_char_p, []),
    "sarbp_default_tuning": (C.c_int, [C.POINTER(Tuning)]),
    "sarbp_focus_fp64": (C.c_int, [C.POINTER(Scene), _P, _P, _P, _P]),
    "sarbp_mixed_workspace_size": (C.c_int64, [C.POINTER(Scene), C.POINTER(Tuning)]),
    "sarbp_focus_mixed": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, _P, _P, _P, _P,
                                    C.c_size_t, _P]),
    "sarbp_mixed_prepare": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, C.c_size_t, _P]),
    "sarbp_focus_mixed_prepared": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, _P, _P,
                                             _P, _P, C.c_size_t, _P]),
    "sarbp_probe_issue_rates": (C.c_int, [C.POINTER(C.c_double), _P]),
    "sarbp_mixed_status": (C.c_int, [_P, C.c_size_t, _P]),
    "sarbp_queue_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(Tuning), C.c_int32,
                                     C.c_int64]),
    "sarbp_queue_submit": (C.c_int64, [_P, C.POINTER(Scene), _P]),
    "sarbp_queue_poll": (C.c_int, [_P, C.c_int64]),
    "sarbp_queue_wait": (C.c_int, [_P, C.c_int64]),
    "sarbp_queue_destroy": (C.c_int, [_P]),
    "sarbp_queue_reserve": (C.c_int, [_P, C.c_size_t]),
    "sarbp_queue_job_bytes": (C.c_int64, [_P, C.POINTER(Scene)]),
    "sarbp_queue_submit_host": (C.c_int64, [_P, C.POINTER(Scene), _P]),
    "sarbp_queue_stats": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "sarbp_queue_cancel": (C.c_int, [_P, C.c_int64]),
    "sarbp_queue_completed": (C.c_int64, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                          C.POINTER(C.c_int32), C.c_int64]),
    "sarbp_tile_queue_keys": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, C.c_size_t,
                                        C.POINTER(C.c_uint32), C.c_int64, _P]),
    "sarbp_focus_mixed_range": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, _P, _P, _P,
                                          _P, C.c_size_t, C.c_int64, C.c_int64, _P]),
    "sarbp_raw_bin_range": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, C.c_size_t,
                                      C.POINTER(C.c_int64), _P]),
    "sarbp_raw_bin_range_async": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P,
                                            C.c_size_t, _P, _P]),
    "sarbp_upload_raw_bins": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int64, C.c_int64,
                                        C.c_int64, _P]),
    "sarbp_upload_raw_bins_sm": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int64,
                                           C.c_int64, C.c_int64, _P]),
    "sarbp_copy_to_device_sm": (C.c_int, [_P, _P, C.c_int64, _P]),
    "sarbp_upload_raw_blocks_sm": (C.c_int, [_P, C.c_int64, _P, C.c_int64, C.c_int64, C.c_int64,
                                             _P, C.c_int32, _P, _P, C.c_uint32, C.c_int32, _P]),
    "sarbp_upload_raw_blocks_bound_sm": (C.c_int, [_P, C.c_int64, _P, C.c_int64, _P, _P,
                                                   C.c_int32, _P, _P, C.c_uint32, C.c_int32,
                                                   _P]),
    "sarbp_stream_wait_flag": (C.c_int, [_P, _P, C.c_uint32]),
    "sarbp_stream_wait_supported": (C.c_int, []),
    "sarbp_upload_host_arrays": (C.c_int, [C.c_int32, _P, _P, _P, _P]),
    "sarbp_device_reads_pageable": (C.c_int, []),
    "sarbp_copy_to_host_sm": (C.c_int, [_P, _P, C.c_int64, _P]),
    "sarbp_focus_mixed_noalloc": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, _P, _P,
                                            _P, _P]),
    "sarbp_amplitude_u8": (C.c_int, [_P, C.c_int64, C.c_double, _P, _P, _P, C.c_size_t, _P]),
    "sarbp_tile_count": (C.c_int64, [C.POINTER(Scene), C.POINTER(Tuning)]),
    "sarbp_tile_costs": (C.c_int, [C.POINTER(Scene), C.POINTER(Tuning), _P, _P]),
    "sarbp_batch_workspace_size": (C.c_int64, [C.c_int32, C.c_int64]),
    "sarbp_batch_set_scene": (C.c_int, [_P, C.c_size_t, C.c_int32, C.c_int32, C.POINTER(Scene),
                                        C.POINTER(Tuning), _P, C.c_size_t, _P, _P, _P, _P]),
    "sarbp_batch_set_items": (C.c_int, [_P, C.c_size_t, C.c_int32, _P, C.c_int64, _P]),
    "sarbp_batch_focus": (C.c_int, [_P, C.c_size_t, C.c_int32, C.POINTER(Tuning), C.c_int64,
                                    C.c_int32, _P, _P]),
}

_lock = threading.Lock()
_lib: C.CDLL | None = None


def load(build_if_needed: bool = True) -> C.CDLL:
    """Load (building first if needed) libsarbp.so and bind its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build_library() if build_if_needed else _build.LIB_PATH
        if not path.exists():
            raise RuntimeError(f"libsarbp.so not found at {path}; run build_library()")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    msg = load().sarbp_last_error()
    return msg.decode() if msg else ""


def check(status: int) -> int:
    """Raise SarbpError for a negative status; return it otherwise."""
    if status < 0:
        raise SarbpError(int(status), last_error())
    return status


def default_tuning() -> Tuning:
    t = Tuning()
    check(load().sarbp_default_tuning(C.byref(t)))
    return t
