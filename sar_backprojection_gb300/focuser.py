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
from .scene import DeviceScene, _pulse_major_host, scene_to_device

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
                         raw_bins=(scene.bin_lo, scene.bin_hi), streamed=True)
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
# how the streamed drop-in copies the reachable raw bins from page-locked
# host memory: "sm" (SM loads of 16-byte words, one CTA per SM, on a stream of
# the highest priority, so its CTAs take SMs as focusing CTAs finish) or
# "copy" (copy engine).  Measured over 240 calls each on the full workload:
# SM loads 3.89 ms mean, 3.85 ms median, 4.09 ms at the 99th percentile; the
# copy engine 4.17 ms mean, 3.41 ms median, 9.5 ms at the 99th percentile and
# 86 ms worst (its host-to-device stalls).  "signal": one persistent copy
# kernel of SIGNAL_CTAS CTAs that sets a device flag per finished block, each
# focusing segment's stream held behind its flag; over 200 calls 3.89 ms mean
# at 64 CTAs (16: 5.97, 32: 4.23, 96: 4.28, 152: 5.03 ms; fewer CTAs cannot
# keep the host link busy, more take SMs from focusing), a tie with "sm"
STREAM_UPLOAD = "sm"
SIGNAL_CTAS = 64       # "signal": CTAs of the persistent block-copy kernel
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
        self.raw: dict[tuple, torch.Tensor] = {}
        self.out: dict[int, torch.Tensor] = {}
        self.images = FreshImages()

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
    ``blocks`` pulse blocks on a copy stream, and after each block the
    queue items whose pulses are all resident are focused on the compute
    stream.  Returns (image, scene).
    """
    lib = _lib.load()
    tq = _lib.Tuning.from_buffer_copy(t)
    tq.staged = 3
    dev = (torch.device(device) if device is not None
           else torch.device("cuda", torch.cuda.current_device()))
    res_cache = _dropin_for(dev)
    with res_cache.lock:
        return _focus_streamed_locked(args, tq, dev, blocks, lib, res_cache)


def _focus_streamed_locked(args, tq, dev, blocks, lib, res_cache: _DropIn):
    nra, naz = (int(v) for v in tuple(args[8].shape))
    scene = scene_to_device(*args, device=dev, raw_bins="bound", tuning=tq,
                            raw_buffer=res_cache.raw_buffer(nra, naz, dev))
    compute = torch.cuda.current_stream(dev)
    sc = C.byref(scene.struct())
    ws = scene.workspace
    nt = _lib.check(int(lib.sarbp_tile_count(sc, C.byref(tq))))
    keys = np.empty(nt, dtype=np.uint32)
    _lib.check(lib.sarbp_tile_queue_keys(sc, C.byref(tq), ws.data_ptr(), ws.numel(),
                                         keys.ctypes.data_as(C.POINTER(C.c_uint32)), nt,
                                         compute.cuda_stream))
    out = res_cache.out_buffer(scene.npix, dev)
    lo, hi = scene.bin_lo, scene.bin_hi
    naz = scene.naz
    # equal pulse blocks, the last one split in two: the tiles that end in
    # the final block are the only work left after the copies, so it is small
    marks = [naz * (k + 1) // blocks for k in range(blocks - 1)]
    marks += [naz - naz // (2 * blocks), naz]
    ends = np.searchsorted(keys, np.asarray(marks, dtype=np.int64), side="right")
    ends[-1] = nt
    pinned = scene.host_rows.is_pinned()
    sm = STREAM_UPLOAD in ("sm", "signal") and pinned
    signal = (STREAM_UPLOAD == "signal" and pinned and hi >= lo and len(marks) <= 32
              and scene.nra % 2 == 0 and scene.pitch % 2 == 0
              and scene.host_rows.data_ptr() % 16 == 0 and scene.raw.data_ptr() % 16 == 0)
    copy = res_cache.copy_sm if sm else res_cache.copy
    upload = lib.sarbp_upload_raw_bins_sm if sm else lib.sarbp_upload_raw_bins
    copy.wait_stream(compute)               # raw buffer and tables allocated on compute
    # segments alternate between two compute streams so that one segment's
    # last CTAs overlap the next segment's first
    side = res_cache.side
    side.wait_stream(compute)
    ws.record_stream(side)
    lanes = (compute, side)
    row = scene.pitch * 8
    first = 0
    a0 = 0
    if signal:
        # one persistent copy kernel on SIGNAL_CTAS SMs; each segment's stream
        # waits for its block's flag, so focusing runs beside the copy
        res_cache.generation = res_cache.generation % 0xFFFFFFFF + 1
        gen = res_cache.generation
        block_ends = np.asarray(marks, dtype=np.int64)
        _lib.check(lib.sarbp_upload_raw_blocks_sm(
            scene.raw.data_ptr(), scene.pitch, scene.host_rows.data_ptr(), scene.nra, lo,
            hi - lo + 1, block_ends.ctypes.data, len(marks), res_cache.flags.data_ptr(),
            res_cache.counters.data_ptr(), gen, SIGNAL_CTAS, copy.cuda_stream))
        scene.h2d_bytes += (hi - lo + 1) * naz * 8
        for k in range(len(marks)):
            lane = lanes[k % 2]
            _lib.check(lib.sarbp_stream_wait_flag(lane.cuda_stream,
                                                  res_cache.flags.data_ptr() + 4 * k, gen))
            count = int(ends[k]) - first
            if count > 0:
                _lib.check(lib.sarbp_focus_mixed_range(sc, C.byref(tq), out.data_ptr(), None,
                                                       None, None, ws.data_ptr(), ws.numel(),
                                                       first, count, lane.cuda_stream))
            first = int(ends[k])
        marks = []                                  # nothing left for the loop below
        compute.wait_stream(copy)
    for k in range(len(marks)):
        a1 = marks[k]
        if hi >= lo and a1 > a0:
            _lib.check(upload(
                scene.raw.data_ptr() + a0 * row, scene.pitch,
                scene.host_rows.data_ptr() + a0 * scene.nra * 8, scene.nra, lo, hi - lo + 1,
                a1 - a0, copy.cuda_stream))
            scene.h2d_bytes += (hi - lo + 1) * (a1 - a0) * 8
        ev = torch.cuda.Event()
        ev.record(copy)
        lane = lanes[k % 2]
        lane.wait_event(ev)
        count = int(ends[k]) - first
        if count > 0:
            _lib.check(lib.sarbp_focus_mixed_range(sc, C.byref(tq), out.data_ptr(), None, None,
                                                   None, ws.data_ptr(), ws.numel(), first,
                                                   count, lane.cuda_stream))
        first = int(ends[k])
        a0 = a1
    compute.wait_stream(side)
    res = FocusResult(image=out, workspace=ws)
    img = res_cache.images.get(scene.dim0, scene.dim1)
    # column-major pixels: the F-order array's memory is the device image's
    dst = torch.from_numpy(img.reshape(-1, order="F").view(np.float64)).view(-1, 2)
    dst.copy_(out)
    del dst
    res.check()
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
