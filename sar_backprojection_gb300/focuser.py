"""Focusing calls: the drop-in for the reference's focusing functions.

``FocalizzatoreBpPx`` keeps the reference's 13 positional arguments, their
meaning and dtype coercions, its ValueErrors and its return value (a fresh
complex128 array of xxg1's shape) -- sar_focuser_puntual_noui.py:149-284.
``FocalizzatoreBpCuPy`` and ``FocalizzatoreBpCuPy_Batched`` are the same call
under the GPU scripts' names (gpu_small_dataset.py:113, :229).  Focusing runs
on the GPU through libsarbp.so; there is no CPU path.

Keyword-only extras: ``precision`` ("fp64", the reference semantics exactly,
or "mixed", the mixed-precision kernel), ``tuning`` and ``device``.  The
reference's progress prints and its ``focalizador_px_checkpoint.npz`` file are
not reproduced: a full scene focuses in milliseconds on one GB300, so the
checkpoint has nothing to resume (long scenes use ``large_scene``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .scene import (DeviceScene, _bound_reached_bins_async, _pulse_major_host,
                    read_bound, scene_to_device)

PRECISIONS = ("fp64", "mixed")


@dataclass
class FocusResult:
    """Device outputs of one focusing call."""

    image: torch.Tensor                    # (npix, 2) float64, column-major pixels
    nvalid: torch.Tensor | None = None     # (npix,) int32 contributor counts
    checksum: torch.Tensor | None = None   # (npix,) int64 (bit pattern of uint64)
    counters: torch.Tensor | None = None   # (NUM_COUNTERS,) int64
    workspace: torch.Tensor | None = None  # mixed: the workspace the kernels ran on

    def status(self) -> int:
        """Mixed path: SARBP_ETIMEOUT if a bounded device wait gave up (the image
        is then incomplete), else SARBP_OK; synchronises the current stream and
        clears the status.  Always SARBP_OK for the FP64 kernel."""
        if self.workspace is None:
            return _lib.SARBP_OK
        return int(_lib.load().sarbp_mixed_status(self.workspace.data_ptr(),
                                                  self.workspace.numel(),
                                                  _stream_ptr(self.workspace.device)))

    def check(self) -> "FocusResult":
        """Raise SarbpError when status() is not SARBP_OK."""
        _lib.check(self.status())
        return self

    def to_numpy(self, dim0: int, dim1: int) -> np.ndarray:
        """complex128 image of shape (dim0, dim1), as the reference returns it."""
        flat = self.image.cpu().numpy().view(np.complex128).reshape(-1)
        return np.reshape(flat, (dim0, dim1), order="F")


def _stream_ptr(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def resolve_tuning(tuning) -> _lib.Tuning:
    t = _lib.default_tuning()
    if tuning is None:
        return t
    if isinstance(tuning, _lib.Tuning):
        return tuning
    for k, v in dict(tuning).items():
        setattr(t, k, int(v))
    return t


def workspace_bytes(scene: DeviceScene, tuning=None) -> int:
    t = resolve_tuning(tuning)
    return _lib.check(int(_lib.load().sarbp_mixed_workspace_size(C.byref(scene.struct()),
                                                                  C.byref(t))))


def focus(scene: DeviceScene, precision: str = "fp64", *, tuning=None,
          out: torch.Tensor | None = None, diagnostics: bool = False,
          workspace: torch.Tensor | None = None) -> FocusResult:
    """Focus a device-resident scene, stream-ordered on torch's current stream.

    ``diagnostics`` also returns per-pixel contributor counts, the (pulse,
    bin) checksum and, for "mixed", the kernel counters.
    """
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    lib = _lib.load()
    dev = scene.device
    if out is None:
        out = torch.empty((scene.npix, 2), dtype=torch.float64, device=dev)
    res = FocusResult(image=out)
    nv_ptr = cs_ptr = ctr_ptr = None
    if diagnostics:
        res.nvalid = torch.empty(scene.npix, dtype=torch.int32, device=dev)
        res.checksum = torch.empty(scene.npix, dtype=torch.int64, device=dev)
        nv_ptr, cs_ptr = res.nvalid.data_ptr(), res.checksum.data_ptr()
    stream = _stream_ptr(dev)
    sc = C.byref(scene.struct())
    if precision == "fp64":
        _lib.check(lib.sarbp_focus_fp64(sc, out.data_ptr(), nv_ptr, cs_ptr, stream))
        return res
    t = resolve_tuning(tuning)
    need = _lib.check(int(lib.sarbp_mixed_workspace_size(sc, C.byref(t))))
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=dev)
    if diagnostics:
        res.counters = torch.zeros(_lib.NUM_COUNTERS, dtype=torch.int64, device=dev)
        ctr_ptr = res.counters.data_ptr()
    _lib.check(lib.sarbp_focus_mixed(sc, C.byref(t), out.data_ptr(), nv_ptr, cs_ptr, ctr_ptr,
                                     workspace.data_ptr(), workspace.numel(), stream))
    res.workspace = workspace
    return res


# bytes moved and raw bins uploaded by the last FocalizzatoreBpPx call
last_call: dict = {}


def FocalizzatoreBpPx(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                      near_range, dra, lambda_val, Sint, *, precision: str = "fp64",
                      tuning=None, device=None) -> np.ndarray:
    """Focus one scene; returns complex128 of xxg1's shape (column-major pixels).

    Drop-in for sar_focuser_puntual_noui.py:149 (same positional arguments).
    Host raw data in the reference's column-major layout are uploaded only
    over the range bins the apertures can reach; with ``precision="mixed"``
    and a staged tuning the upload is streamed in pulse blocks and focusing
    overlaps it (tiles run as soon as the pulses up to their last one are
    resident).  The image is the same either way.
    """
    t = resolve_tuning(tuning)
    if precision == "mixed" and t.staged and _pulse_major_host(Raw_Data) is not None:
        img, scene = _focus_streamed((xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz,
                                      Raw_Data, near_range, dra, lambda_val, Sint), t, device)
        last_call.update(h2d_bytes=scene.h2d_bytes, d2h_bytes=img.nbytes,
                         raw_bins=(scene.bin_lo, scene.bin_hi), streamed=True,
                         upload=scene.upload,
                         small_upload=getattr(scene, "small_upload", "per-array"),
                         d2h=scene.d2h, launches=scene.launches)
        return img
    scene = scene_to_device(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                            near_range, dra, lambda_val, Sint, device=device, raw_bins="reached")
    res = focus(scene, precision, tuning=t, workspace=scene.workspace)
    img = res.to_numpy(scene.dim0, scene.dim1)
    last_call.update(h2d_bytes=scene.h2d_bytes, d2h_bytes=img.nbytes,
                     raw_bins=(scene.bin_lo, scene.bin_hi), streamed=False)
    res.check()          # a device wait that gave up leaves an incomplete image
    return img


STREAM_BLOCKS = 8      # pulse blocks of a streamed drop-in upload
# the final block is halved STREAM_TAIL times: the tiles whose apertures end
# in the last pulses (all those clipped at the scene's end) wait for the
# final rows, so the last blocks are kept short
STREAM_TAIL = 3
STREAM_HEAD = 2        # halvings of the first block (3.473 vs 3.484 ms: within noise)
STREAM_LANES = 3       # compute streams the focusing segments rotate over
# "one-call": the DEM, masks and trajectory go up in one foreign call when
# their dtypes and layout need no conversion; "torch": per-array copies
SMALL_UPLOAD = "one-call"
# How the streamed drop-in copies the reachable raw bins from page-locked
# host memory.  "signal" (default): the host does not wait for the bin bound;
# one persistent copy kernel of SIGNAL_CTAS CTAs (four rows, 64 KB of loads
# in flight per CTA) reads the bound, copies the blocks in order and sets a
# device flag per finished block, and each focusing segment's stream is held
# behind its block's flag.  "sm": per-block SM-load copies (one CTA per SM,
# highest-priority stream) after a host wait for the bound.  "copy": the
# copy engine per block.  Pageable raw rows always take the copy engine.
# Full workload, 200 calls each, one run: "signal" 3.52 ms mean, 3.54 ms at
# the 99th percentile (24 CTAs 3.69, 32: 3.55, 48: 3.57); "sm" 3.99 / 4.31;
# the copy engine's median is 3.41 ms but it stalls for tens of ms now and
# then (p99 9.5 ms, worst 86 ms in an earlier run).
STREAM_UPLOAD = "signal"
SIGNAL_CTAS = 40       # "signal": CTAs of the persistent block-copy kernel
FRESH_AHEAD = 2        # result arrays the drop-in call keeps faulted in ahead


class FreshImages:
    """The complex128 (dim0, dim1) column-major host arrays the drop-in call
    returns: each call gets a NEW array, as the reference's focusing call
    returns one, whose pages a helper thread has already touched.  A fresh
    16 MB result would otherwise cost thousands of page faults inside the
    call.  The helper keeps up to FRESH_AHEAD arrays of the last shape asked
    for; a call that finds none ready allocates one itself."""

    def __init__(self, ahead: int = FRESH_AHEAD):
        import threading
        self.ahead = int(ahead)
        self.ready: list = []                 # (shape, tensor) faulted in
        self.shape = None
        self.cv = threading.Condition()
        self.thread = None

    @staticmethod
    def _make(dim0: int, dim1: int) -> torch.Tensor:
        t = torch.empty((dim0 * dim1, 2), dtype=torch.float64)
        t.zero_()                              # touches every page, interpreter lock released
        return t

    def _fill(self):
        while True:
            with self.cv:
                while self.shape is None or len(self.ready) >= self.ahead:
                    self.cv.wait()
                shape = self.shape
            t = self._make(*shape)
            with self.cv:
                if shape == self.shape and len(self.ready) < self.ahead:
                    self.ready.append((shape, t))

    def get(self, dim0: int, dim1: int) -> np.ndarray:
        import threading
        shape = (int(dim0), int(dim1))
        t = None
        with self.cv:
            if self.shape != shape:
                self.shape = shape
                self.ready.clear()
            if self.ready:
                t = self.ready.pop()[1]
            if self.thread is None:
                self.thread = threading.Thread(target=self._fill, daemon=True)
                self.thread.start()
            self.cv.notify()
        if t is None:
            t = self._make(*shape)
        # the array's memory is the tensor's; the array keeps it alive
        flat = t.numpy().view(np.complex128).reshape(-1)
        return np.reshape(flat, shape, order="F")

    def clear(self) -> None:
        with self.cv:
            self.ready.clear()


class _DropIn:
    """Per-device resources the synchronous drop-in call reuses across calls:
    its copy and second compute stream, device buffers for the raw rows and
    the image (a caller's repeated calls then allocate nothing on the device)
    and the pre-faulted fresh host images it returns.  The lock serialises calls from
    several host threads."""

    def __init__(self, dev: torch.device):
        import threading
        self.lock = threading.Lock()
        self.copy = torch.cuda.Stream(dev)
        self.copy_sm = torch.cuda.Stream(dev, priority=torch.cuda.Stream.priority_range()[1])
        # "signal" uploads: per-block flags (never cleared: each call waits
        # for its own generation) and the copy kernel's block counters
        self.flags = torch.zeros(32, dtype=torch.int32, device=dev)
        self.counters = torch.zeros(32, dtype=torch.int32, device=dev)
        self.generation = 0
        self.side = torch.cuda.Stream(dev)
        self.side2 = torch.cuda.Stream(dev)
        self.bound_host = torch.zeros(2, dtype=torch.int32).pin_memory()
        self.raw: dict[tuple, torch.Tensor] = {}
        self.out: dict[int, torch.Tensor] = {}
        self.small: dict[tuple, tuple] = {}
        self.images = FreshImages()
        # kernels on this device read and write pageable host memory in place
        with torch.cuda.device(dev):
            self.pageable = bool(_lib.load().sarbp_device_reads_pageable())
        # "signal" uploads need the driver's stream wait on a memory value
        self.wait_ok = bool(_lib.load().sarbp_stream_wait_supported())

    def small_buffers(self, npix: int, naz: int, dev) -> tuple:
        """One device buffer for the DEM, masks and trajectory of a scene
        shape: (views by DeviceScene field name, device addresses, bytes)."""
        key = (npix, naz)
        if key not in self.small:
            self.small.clear()
            sizes = [npix * 8] * 3 + [npix, npix * 4, npix * 4] + [naz * 8] * 3
            offs, o = [], 0
            for b in sizes:
                offs.append(o)
                o += -(-b // 256) * 256
            buf = torch.empty(max(o, 1), dtype=torch.uint8, device=dev)
            views = {name: buf[off:off + b].view(dt)
                     for (name, dt), off, b in zip(_SMALL_FIELDS, offs, sizes)}
            dptrs = (C.c_void_p * 9)(*[views[n].data_ptr() for n, _ in _SMALL_FIELDS])
            self.small[key] = (views, dptrs, (C.c_int64 * 9)(*sizes), sum(sizes))
        return self.small[key]

    def raw_buffer(self, nra: int, naz: int, dev) -> torch.Tensor:
        key = (naz, nra + (nra & 1))
        if key not in self.raw:
            self.raw.clear()                   # one scene shape at a time
            self.raw[key] = torch.empty((naz, key[1], 2), dtype=torch.float32, device=dev)
        return self.raw[key]

    def out_buffer(self, npix: int, dev) -> torch.Tensor:
        if npix not in self.out:
            self.out.clear()
            self.out[npix] = torch.empty((npix, 2), dtype=torch.float64, device=dev)
        return self.out[npix]


_dropin: dict = {}


def release_drop_in_buffers() -> None:
    """Free the device buffers the drop-in call keeps between calls."""
    for r in _dropin.values():
        with r.lock:
            r.raw.clear()
            r.out.clear()
            r.small.clear()
            r.images.clear()


def _dropin_for(dev: torch.device) -> _DropIn:
    key = (dev.type, dev.index)
    if key not in _dropin:
        _dropin[key] = _DropIn(dev)
    return _dropin[key]


def _focus_streamed(args, t: _lib.Tuning, device, blocks: int = STREAM_BLOCKS):
    """Drop-in focusing with the raw upload overlapped by focusing.

    The queue of the scene's tiles is ordered by last aperture pulse
    (staged=3); the reachable range bins of the pulse rows go up in
    ``blocks`` pulse blocks (the last one halved STREAM_TAIL times) on a copy
    stream, and after each block the queue items whose pulses are all
    resident are focused, the segments rotating over STREAM_LANES streams.
    With STREAM_UPLOAD "signal" and page-locked raw rows the small inputs go
    up in one call, the host never waits for the bin bound, and the blocks
    come from one persistent copy kernel whose per-block device flags the
    segments' streams wait on.  Returns (image, scene).
    """
    lib = _lib.load()
    tq = _lib.Tuning.from_buffer_copy(t)
    tq.staged = 3
    dev = (torch.device(device) if device is not None
           else torch.device("cuda", torch.cuda.current_device()))
    res_cache = _dropin_for(dev)
    with res_cache.lock:
        return _focus_streamed_locked(args, tq, dev, blocks, lib, res_cache)


# DeviceScene fields held in the drop-in's small-array buffer, in order
_SMALL_FIELDS = (("x", torch.float64), ("y", torch.float64), ("z", torch.float64),
                 ("mask", torch.uint8), ("index", torch.int32), ("sint", torch.int32),
                 ("tx", torch.float64), ("ty", torch.float64), ("tz", torch.float64))
_NP_OF = {torch.float64: np.dtype(np.float64), torch.uint8: np.dtype(np.uint8),
          torch.int32: np.dtype(np.int32)}


def _file_backed(a) -> bool:
    """Whether an array's memory is a file mapping (np.memmap, mmap): kernels
    reading it in place would fault its pages in from the GPU one by one, so
    such arrays take the driver's staged copies (CPU page-ins, readahead)."""
    import mmap
    seen = 0
    while a is not None and seen < 32:
        if isinstance(a, (np.memmap, mmap.mmap)):
            return True
        a = getattr(a, "base", None)
        seen += 1
    return False


def _column_major_words(a, dt: torch.dtype, n: int, exact: bool):
    """Host address of an array of dtype ``dt`` whose column-major flatten
    (the reference's ``flatten(order='F')``) is its memory order, with n
    elements (at least n unless ``exact``); None otherwise."""
    if isinstance(a, np.ndarray):
        if (a.dtype != _NP_OF[dt] or not a.flags.f_contiguous
                or (a.size != n if exact else a.size < n) or _file_backed(a)):
            return None
        return a.__array_interface__["data"][0]
    if isinstance(a, torch.Tensor):
        if (a.device.type != "cpu" or a.dtype != dt
                or (a.numel() != n if exact else a.numel() < n)):
            return None
        expect = 1
        for size, stride in zip(a.shape, a.stride()):
            if size != 1 and stride != expect:
                return None
            expect *= size
        return a.data_ptr()
    return None


def _scene_from_host(args, dev, lib, res_cache: _DropIn, raw_buffer, host_rows):
    """The drop-in's DeviceScene without per-array Python work: when every
    DEM, mask and trajectory argument already has the dtype the reference
    casts it to and column-major memory order, all nine go up in one
    sarbp_upload_host_arrays call into the per-shape buffer.  None when an
    argument needs a cast, a copy or a check (scene_to_device does those)."""
    (xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, raw, near_range, dra, lambda_val,
     sint) = args
    if len(tuple(xxg1.shape)) != 2:
        return None
    dim0, dim1 = (int(v) for v in xxg1.shape)
    npix = dim0 * dim1
    nra, naz = (int(v) for v in raw.shape)
    srcs = []
    for a, (_, dt) in zip((xxg1, yyg1, zzg1, mask, index, sint), _SMALL_FIELDS):
        srcs.append(_column_major_words(a, dt, npix, True))
    for w in (wgsx, wgsy, wgsz):
        srcs.append(_column_major_words(w, torch.float64, naz, False))
    if any(p is None for p in srcs):
        return None
    views, dptrs, sizes, total = res_cache.small_buffers(npix, naz, dev)
    _lib.check(lib.sarbp_upload_host_arrays(9, dptrs, (C.c_void_p * 9)(*srcs), sizes,
                                            torch.cuda.current_stream(dev).cuda_stream))
    scene = DeviceScene(dim0=dim0, dim1=dim1, raw=raw_buffer, nra=nra, naz=naz,
                        pitch=nra + (nra & 1), near_range=float(near_range),
                        delta_range=float(dra), lambda_=float(lambda_val),
                        **{name: views[name] for name, _ in _SMALL_FIELDS})
    scene.h2d_bytes = total
    scene.host_rows = host_rows
    scene.small_upload = "one-call"
    # copy kernels among the nine copies (the rest went through the driver)
    scene.small_kernels = 9 if res_cache.pageable else sum(
        1 for a in (xxg1, yyg1, zzg1, mask, index, sint, wgsx, wgsy, wgsz)
        if isinstance(a, torch.Tensor) and a.is_pinned())
    return scene


def _stream_marks(naz: int, blocks: int, tail: int, head: int = 0) -> list[int]:
    """Pulse block ends: ``blocks`` equal blocks, the first one halved
    ``head`` times (focusing starts on a short first block) and the last one
    halved ``tail`` times (at most 32 ends)."""
    marks = [naz // (blocks << h) for h in range(head, 0, -1)]
    marks += [naz * (k + 1) // blocks for k in range(blocks - 1)]
    for h in range(1, tail + 1):
        marks.append(naz - naz // (blocks << h))
    marks.append(naz)
    return marks[-32:] if len(marks) > 32 else marks


def _focus_streamed_locked(args, tq, dev, blocks, lib, res_cache: _DropIn):
    nra, naz = (int(v) for v in tuple(args[8].shape))
    host_rows = _pulse_major_host(args[8])
    # "signal": the bound is not waited for; the persistent block copy reads
    # it from page-locked memory once the stream has computed it
    # rows kernels can load: page-locked, or pageable on a device that reads
    # it in place (not a file mapping: see _file_backed)
    reachable = host_rows is not None and (
        host_rows.is_pinned() or (res_cache.pageable and not _file_backed(args[8])))
    signal = (STREAM_UPLOAD == "signal" and res_cache.wait_ok and reachable and nra % 2 == 0
              and host_rows.data_ptr() % 16 == 0)
    raw_buffer = res_cache.raw_buffer(nra, naz, dev)
    if not signal:
        scene = scene_to_device(*args, device=dev, raw_bins="bound", tuning=tq,
                                raw_buffer=raw_buffer)
    else:
        scene = None
        if SMALL_UPLOAD == "one-call":
            scene = _scene_from_host(args, dev, lib, res_cache, raw_buffer, host_rows)
        if scene is None:
            scene = scene_to_device(*args, device=dev, raw_bins="deferred", tuning=tq,
                                    raw_buffer=raw_buffer, bound_host=res_cache.bound_host)
        else:
            _bound_reached_bins_async(scene, res_cache.bound_host, tuning=tq)
    compute = torch.cuda.current_stream(dev)
    sc = C.byref(scene.struct())
    ws = scene.workspace
    marks = _stream_marks(scene.naz, blocks, STREAM_TAIL, STREAM_HEAD)
    side, side2 = res_cache.side, res_cache.side2
    lanes = (compute, side, side2)[:max(1, min(3, STREAM_LANES))]
    for lane in lanes[1:]:
        lane.wait_stream(compute)
        ws.record_stream(lane)
    out = res_cache.out_buffer(scene.npix, dev)
    if signal:
        copy = res_cache.copy_sm
        copy.wait_stream(compute)           # bound, raw buffer and tables on compute
        res_cache.generation = res_cache.generation % 0xFFFFFFFF + 1
        gen = res_cache.generation
        block_ends = np.asarray(marks, dtype=np.int64)
        _lib.check(lib.sarbp_upload_raw_blocks_bound_sm(
            scene.raw.data_ptr(), scene.pitch, host_rows.data_ptr(), nra,
            res_cache.bound_host.data_ptr(), block_ends.ctypes.data, len(marks),
            res_cache.flags.data_ptr(), res_cache.counters.data_ptr(), gen, SIGNAL_CTAS,
            copy.cuda_stream))
    nt = _lib.check(int(lib.sarbp_tile_count(sc, C.byref(tq))))
    keys = np.empty(nt, dtype=np.uint32)
    _lib.check(lib.sarbp_tile_queue_keys(sc, C.byref(tq), ws.data_ptr(), ws.numel(),
                                         keys.ctypes.data_as(C.POINTER(C.c_uint32)), nt,
                                         compute.cuda_stream))
    ends = np.searchsorted(keys, np.asarray(marks, dtype=np.int64), side="right")
    ends[-1] = nt
    if signal:
        lo, hi = read_bound(scene)           # the keys' synchronisation passed the bound
    else:
        lo, hi = scene.bin_lo, scene.bin_hi
        sm = STREAM_UPLOAD in ("sm", "signal") and reachable
        copy = res_cache.copy_sm if sm else res_cache.copy
        upload = lib.sarbp_upload_raw_bins_sm if sm else lib.sarbp_upload_raw_bins
        copy.wait_stream(compute)           # raw buffer and tables allocated on compute
    row = scene.pitch * 8
    first = 0
    a0 = 0
    # this library's kernels the call launches: chunk tables, the bound (3),
    # the queue keys, the small-input copies, then per block below
    launches = 1 + 3 + 1 + getattr(scene, "small_kernels", 0) + (1 if signal else 0)
    for k in range(len(marks)):
        a1 = marks[k]
        lane = lanes[k % len(lanes)]
        if signal:
            # each segment's stream waits for its block's flag, so focusing
            # runs beside the copy kernel
            _lib.check(lib.sarbp_stream_wait_flag(lane.cuda_stream,
                                                  res_cache.flags.data_ptr() + 4 * k, gen))
        else:
            if hi >= lo and a1 > a0:
                _lib.check(upload(
                    scene.raw.data_ptr() + a0 * row, scene.pitch,
                    scene.host_rows.data_ptr() + a0 * scene.nra * 8, scene.nra, lo,
                    hi - lo + 1, a1 - a0, copy.cuda_stream))
                launches += 1 if sm else 0
            ev = torch.cuda.Event()
            ev.record(copy)
            lane.wait_event(ev)
        count = int(ends[k]) - first
        if count > 0:
            _lib.check(lib.sarbp_focus_mixed_range(sc, C.byref(tq), out.data_ptr(), None, None,
                                                   None, ws.data_ptr(), ws.numel(), first,
                                                   count, lane.cuda_stream))
            launches += 1
        first = int(ends[k])
        a0 = a1
    if hi >= lo:
        scene.h2d_bytes += (hi - lo + 1) * naz * 8
    scene.upload = "signal" if signal else ("sm" if sm else "copy")
    for lane in lanes[1:]:
        compute.wait_stream(lane)
    compute.wait_stream(copy)
    res = FocusResult(image=out, workspace=ws)
    img = res_cache.images.get(scene.dim0, scene.dim1)
    # column-major pixels: the F-order array's memory is the device image's
    if res_cache.pageable:
        # SM stores straight into the fresh array, in stream order
        _lib.check(lib.sarbp_copy_to_host_sm(img.__array_interface__["data"][0],
                                             out.data_ptr(), img.nbytes, compute.cuda_stream))
        scene.d2h = "sm"
        launches += 1
    else:
        dst = torch.from_numpy(img.reshape(-1, order="F").view(np.float64)).view(-1, 2)
        dst.copy_(out)
        del dst
        scene.d2h = "copy"
    res.check()                              # synchronises the stream
    scene.launches = launches
    return img, scene


def FocalizzatoreBpCuPy(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                        near_range, dra, lambda_val, Sint, **kw) -> np.ndarray:
    """Same call under gpu_small_dataset.py:113's name."""
    return FocalizzatoreBpPx(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                             near_range, dra, lambda_val, Sint, **kw)


def FocalizzatoreBpCuPy_Batched(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                                near_range, dra, lambda_val, Sint, batch_size=500000,
                                **kw) -> np.ndarray:
    """Same call under gpu_small_dataset.py:229's name.

    ``batch_size`` (pixels per launch in the reference, a memory limit of
    24 GB cards) is accepted and checked but the scene is focused in one
    launch: the per-batch host round trips are what this focuser removes.
    """
    if int(batch_size) <= 0:
        raise ValueError("batch_size must be positive")
    return FocalizzatoreBpPx(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                             near_range, dra, lambda_val, Sint, **kw)
