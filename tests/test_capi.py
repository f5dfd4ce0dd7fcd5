"""The C-ABI library builds, loads and exports what include/*.h declares.

CPU-only: only calls that fail argument validation before touching CUDA are
made here.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

from sar_backprojection_gb300 import _lib
from sar_backprojection_gb300 import build as sbuild

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = h.read_text()
        names.update(re.findall(r"SARBP_API\s+[\w\s\*]+?\b(sarbp_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "sarbp_focus_fp64" in syms and "sarbp_focus_mixed" in syms
    assert len(syms) >= 6


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(sbuild.build_library()))
    for name in declared_symbols():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_python_binding_covers_header():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_struct_layout_matches_header():
    # sarbp_scene: 2 int64 + 10 pointers + 3 int64 + 3 doubles
    assert C.sizeof(_lib.Scene) == 8 * (2 + 10 + 3 + 3)
    assert C.sizeof(_lib.Tuning) == 4 * 8


def test_version_and_defaults():
    lib = _lib.load()
    assert lib.sarbp_version() >= 100
    t = _lib.default_tuning()
    assert t.chunk in (32, 64) and t.tile0 > 0 and t.tile1 > 0


def test_null_scene_is_rejected_with_message():
    lib = _lib.load()
    rc = lib.sarbp_focus_fp64(None, None, None, None, None)
    assert rc == _lib.SARBP_EINVAL
    assert "NULL" in _lib.last_error()
    with pytest.raises(_lib.SarbpError):
        _lib.check(rc)


def test_bad_shapes_are_rejected():
    lib = _lib.load()
    s = _lib.Scene()
    s.dim0, s.dim1 = 4, 4
    for f in ("dem_x", "dem_y", "dem_z", "mask", "index", "sint", "traj_x", "traj_y",
              "traj_z", "raw"):
        setattr(s, f, 0x1000)                  # never dereferenced: validation fails first
    s.nra, s.naz, s.raw_pitch = 8, 16, 4      # pitch < nra
    s.delta_range, s.lambda_ = 0.5, 0.031
    out = C.c_void_p(0x2000)
    assert lib.sarbp_focus_fp64(C.byref(s), out, None, None, None) == _lib.SARBP_EINVAL
    assert "raw_pitch" in _lib.last_error()
    s.raw_pitch = 8
    s.delta_range = 0.0
    assert lib.sarbp_focus_fp64(C.byref(s), out, None, None, None) == _lib.SARBP_EINVAL
    s.delta_range = 0.5
    s.dim0 = 0
    assert lib.sarbp_focus_fp64(C.byref(s), out, None, None, None) == _lib.SARBP_EINVAL


def test_workspace_size_is_host_only():
    lib = _lib.load()
    s = _lib.Scene()
    s.dim0, s.dim1 = 4000, 250
    for f in ("dem_x", "dem_y", "dem_z", "mask", "index", "sint", "traj_x", "traj_y",
              "traj_z", "raw"):
        setattr(s, f, 0x1000)
    s.nra, s.naz, s.raw_pitch = 4762, 40001, 4762
    s.delta_range, s.lambda_, s.near_range = 0.5, 0.031, 3500.0
    t = _lib.default_tuning()
    assert t.staged == 1
    n = lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t))
    assert n >= 16 * 40001
    t.staged = 2                               # + the tile queue: 4 arrays of 4000 tiles
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) >= n + 16 * 4000
    t.staged = 3                               # queue ordered by last pulse: same size
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) >= n + 16 * 4000
    t.staged = 4
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) == _lib.SARBP_EINVAL
    assert "staged" in _lib.last_error()
    t.staged = 1
    t.withhold = 2                              # diagnostic field: 0 or 1
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) == _lib.SARBP_EINVAL
    t.withhold = 0
    t.wait_polls = -1
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) == _lib.SARBP_EINVAL
    t.wait_polls = 0
    t.chunk = 48
    assert lib.sarbp_mixed_workspace_size(C.byref(s), C.byref(t)) == _lib.SARBP_EINVAL


def test_new_entry_points_reject_bad_arguments_without_a_gpu():
    """Argument checks of the upload, bound, queue-range and serving-queue
    entry points run on the host and never touch a device."""
    lib = _lib.load()
    # upload of a bin range that does not fit the rows
    assert lib.sarbp_upload_raw_bins(C.c_void_p(0x1000), 100, C.c_void_p(0x2000), 100, 90, 20,
                                     5, None) == _lib.SARBP_EINVAL
    assert "bin range" in _lib.last_error()
    assert lib.sarbp_upload_raw_bins(None, 100, C.c_void_p(0x2000), 100, 0, 10, 5,
                                     None) == _lib.SARBP_EINVAL
    # zero bins or pulses: nothing to do
    assert lib.sarbp_upload_raw_bins(C.c_void_p(0x1000), 100, C.c_void_p(0x2000), 100, 0, 0,
                                     5, None) == _lib.SARBP_OK
    # the SM-load variants check the same arguments before touching the GPU
    assert lib.sarbp_upload_raw_bins_sm(C.c_void_p(0x1000), 100, C.c_void_p(0x2000), 100, 90,
                                        20, 5, None) == _lib.SARBP_EINVAL
    assert "bin range" in _lib.last_error()
    assert lib.sarbp_upload_raw_bins_sm(None, 100, C.c_void_p(0x2000), 100, 0, 10, 5,
                                        None) == _lib.SARBP_EINVAL
    assert lib.sarbp_upload_raw_bins_sm(C.c_void_p(0x1000), 100, C.c_void_p(0x2000), 100, 0,
                                        0, 5, None) == _lib.SARBP_OK
    assert lib.sarbp_copy_to_device_sm(None, C.c_void_p(0x2000), 16, None) == _lib.SARBP_EINVAL
    assert lib.sarbp_copy_to_device_sm(C.c_void_p(0x1000), C.c_void_p(0x2000), -1,
                                       None) == _lib.SARBP_EINVAL
    assert lib.sarbp_copy_to_device_sm(C.c_void_p(0x1000), C.c_void_p(0x2000), 0,
                                       None) == _lib.SARBP_OK
    # block-signalled copy: odd pitch, decreasing ends, too many blocks, generation 0
    ends = (C.c_int64 * 40)(*range(1, 41))
    fl, ct = C.c_void_p(0x5000), C.c_void_p(0x6000)
    args = [C.c_void_p(0x1000), 100, C.c_void_p(0x2000), 100, 0, 10, ends, 4, fl, ct, 1, 8,
            None]
    for i, bad in ((1, 101), (3, 99), (5, 101), (7, 33), (7, 0), (10, 0), (11, 0), (0, None)):
        a = list(args)
        a[i] = bad
        assert lib.sarbp_upload_raw_blocks_sm(*a) == _lib.SARBP_EINVAL, (i, bad)
    desc = (C.c_int64 * 3)(5, 3, 9)
    a = list(args)
    a[6], a[7] = desc, 3
    assert lib.sarbp_upload_raw_blocks_sm(*a) == _lib.SARBP_EINVAL
    assert "decrease" in _lib.last_error()
    assert lib.sarbp_upload_raw_blocks_bound_sm(C.c_void_p(0x1000), 100, C.c_void_p(0x2000),
                                                100, None, ends, 4, fl, ct, 1, 8,
                                                None) == _lib.SARBP_EINVAL
    assert lib.sarbp_upload_raw_blocks_bound_sm(C.c_void_p(0x1000), 101, C.c_void_p(0x2000),
                                                100, C.c_void_p(0x7000), ends, 4, fl, ct, 1, 8,
                                                None) == _lib.SARBP_EINVAL
    assert lib.sarbp_stream_wait_flag(None, None, 1) == _lib.SARBP_EINVAL
    # one-call uploads: a negative count, a NULL list or a NULL array with bytes
    assert lib.sarbp_upload_host_arrays(-1, None, None, None, None) == _lib.SARBP_EINVAL
    assert lib.sarbp_upload_host_arrays(2, None, None, None, None) == _lib.SARBP_EINVAL
    dsts = (C.c_void_p * 2)(0x1000, None)
    srcs = (C.c_void_p * 2)(0x2000, 0x3000)
    nbytes = (C.c_int64 * 2)(0, 16)
    assert lib.sarbp_upload_host_arrays(2, dsts, srcs, nbytes, None) == _lib.SARBP_EINVAL
    assert "array 1" in _lib.last_error()
    assert lib.sarbp_upload_host_arrays(0, None, None, None, None) == _lib.SARBP_OK
    s = _lib.Scene()
    s.dim0, s.dim1 = 64, 16
    for f in ("dem_x", "dem_y", "dem_z", "mask", "index", "sint", "traj_x", "traj_y",
              "traj_z", "raw"):
        setattr(s, f, 0x1000)
    s.nra, s.naz, s.raw_pitch = 512, 1201, 512
    s.delta_range, s.lambda_, s.near_range = 0.5, 0.031, 3500.0
    t = _lib.default_tuning()
    rng = (C.c_int64 * 2)()
    # bound without a workspace
    assert lib.sarbp_raw_bin_range(C.byref(s), C.byref(t), None, 0, rng,
                                   None) == _lib.SARBP_EWORKSPACE
    hr = (C.c_int32 * 2)()
    assert lib.sarbp_raw_bin_range_async(C.byref(s), C.byref(t), None, 0, hr,
                                         None) == _lib.SARBP_EWORKSPACE
    assert lib.sarbp_raw_bin_range(C.byref(s), C.byref(t), C.c_void_p(0x4000), 1 << 30,
                                   None, None) == _lib.SARBP_EINVAL
    # queue range / keys need a queued tuning
    out = C.c_void_p(0x3000)
    assert lib.sarbp_focus_mixed_range(C.byref(s), C.byref(t), out, None, None, None,
                                       C.c_void_p(0x4000), 1 << 30, 0, 4,
                                       None) == _lib.SARBP_EINVAL
    keys = (C.c_uint32 * 4)()
    t.staged = 3
    assert lib.sarbp_tile_queue_keys(C.byref(s), C.byref(t), None, 0, keys, 4,
                                     None) == _lib.SARBP_EWORKSPACE
    # serving queue: bad sizes, a non-batch tuning, and a NULL destroy
    q = C.c_void_p()
    assert lib.sarbp_queue_create(C.byref(q), None, 0, 0) == _lib.SARBP_EINVAL
    t2 = _lib.default_tuning()
    t2.staged = 2
    assert lib.sarbp_queue_create(C.byref(q), C.byref(t2), 4, 0) == _lib.SARBP_EINVAL
    assert "staged = 1" in _lib.last_error()
    assert lib.sarbp_queue_submit(None, C.byref(s), out) == _lib.SARBP_EINVAL
    assert lib.sarbp_queue_destroy(None) == _lib.SARBP_OK
    # host-memory jobs: NULL queue / output, nothing to reserve
    assert lib.sarbp_queue_reserve(None, 1 << 20) == _lib.SARBP_EINVAL
    assert lib.sarbp_queue_job_bytes(None, C.byref(s)) == _lib.SARBP_EINVAL
    assert lib.sarbp_queue_submit_host(None, C.byref(s), out) == _lib.SARBP_EINVAL
    ids = (C.c_int64 * 4)()
    assert lib.sarbp_queue_completed(None, ids, None, None, 4) == _lib.SARBP_EINVAL
    assert lib.sarbp_queue_cancel(None, 0) == _lib.SARBP_EINVAL
    assert lib.sarbp_queue_stats(None, ids) == _lib.SARBP_EINVAL
