"""Device-resident large-scene focusing: the chunked-azimuth driver.

Replaces the reference's SARSuperOptimizedFocuser.process_dataset
(main_gpu.py:291-621), which for every 2000-column DEM batch memory-maps a raw
azimuth window (+-100 pulses of overlap), converts it on the host, copies it
to the GPU, launches one kernel per point sub-batch, copies results back,
writes an HDF5 slice and a JSON checkpoint.

Here the raw data (15.4 GB for the reference's 4762 x 403484 example) live in
HBM once: they are streamed from the memory-mapped .dat file through two
pinned staging buffers on a copy stream, and each DEM batch is focused as
soon as the pulses its apertures reach are resident -- one launch per batch,
no host synchronisation between batches (the per-pulse chunk tables are
built once for the whole trajectory).  Results come back through pinned
buffers one batch behind and are written into a memory-mapped complex128
column-major output file; after each batch is written the job cursor
(a small JSON file: scene shape, batch size, next batch) is updated, so an
interrupted run resumes at the first unwritten batch.

The azimuth axis of the DEM grid is its second axis (the reference's
(DimRg, DimAz) layout, main_gpu.py:321-324); batches are column blocks,
which are contiguous in the column-major files.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time
import warnings
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _lib, datfiles
from .focuser import resolve_tuning
from .scene import DeviceScene, flatten_f


@dataclass
class Cursor:
    """Resumable job state, written after each finished batch."""

    dim0: int
    dim1: int
    nra: int
    naz: int
    batch_cols: int
    next_batch: int = 0

    def save(self, path) -> None:
        tmp = Path(str(path) + ".tmp")
        tmp.write_text(json.dumps(self.__dict__))
        os.replace(tmp, path)

    @staticmethod
    def load(path):
        try:
            return Cursor(**json.loads(Path(path).read_text()))
        except (OSError, ValueError, TypeError):
            return None

    def matches(self, other: "Cursor") -> bool:
        return all(getattr(self, k) == getattr(other, k)
                   for k in ("dim0", "dim1", "nra", "naz", "batch_cols"))


def pulse_range_tensor(index: torch.Tensor, sint: torch.Tensor, mask: torch.Tensor,
                       naz: int) -> torch.Tensor:
    """[lo, hi] (int64, on the inputs' device) of the pulses the kept
    apertures of a block of pixels reach; lo > hi when none is kept.  The
    reference's rules: aperture ceil(Sint/2)*2+1 pulses from
    Index - ceil(|Sint|/2), pulses 0 < a < Naz-1, Mask == 1, Sint != -9999
    (sar_focuser_puntual_noui.py:35-55, :195-198)."""
    s = sint.reshape(-1).to(torch.int64)
    idx = index.reshape(-1).to(torch.int64)
    m = mask.reshape(-1)
    if not (s.shape == idx.shape == m.shape):
        raise ValueError("index, sint and mask blocks differ in size")
    off = (s.abs() + 1) >> 1                                  # ceil(|s|/2)
    jj = ((s + 1) >> 1) * 2 + 1                               # ceil(s/2)*2 + 1
    lo = torch.clamp(idx - off, min=1)
    hi = torch.clamp(idx - off + jj - 1, max=naz - 2)
    keep = (m == 1) & (s != -9999) & (jj > 0) & (lo <= hi)
    big = torch.iinfo(torch.int64).max
    return torch.stack([torch.where(keep, lo, big).min(), torch.where(keep, hi, -1).max()])


def batch_pulse_range(index_cols: np.ndarray, sint_cols: np.ndarray, mask_cols: np.ndarray,
                      naz: int) -> tuple[int, int]:
    """[lo, hi] of the pulses the kept apertures of a DEM batch reach, or (0, -1)."""
    def flat(a, dt):
        # any memory order will do: only minima and maxima are taken
        a = np.asarray(a)
        return torch.from_numpy(np.ascontiguousarray(a.astype(dt, copy=False).ravel(order="K")))

    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)      # read-only memory maps
        r = pulse_range_tensor(flat(index_cols, np.int32), flat(sint_cols, np.int32),
                               flat(mask_cols, np.uint8), naz)
    lo, hi = int(r[0]), int(r[1])
    return (lo, hi) if lo <= hi else (0, -1)


def _pread_full(fd: int, mv: memoryview, pos: int) -> None:
    while len(mv):
        k = os.preadv(fd, [mv], pos)
        if k <= 0:
            raise EOFError(f"file ends before byte {pos + len(mv)}")
        mv = mv[k:]
        pos += k


def _pwrite_full(fd: int, mv: memoryview, pos: int) -> None:
    while len(mv):
        k = os.pwrite(fd, mv, pos)
        if k <= 0:
            raise OSError("short write")
        mv = mv[k:]
        pos += k


class FileIO:
    """Positional reads and writes of byte ranges of files, split over a
    thread pool (the system calls release the interpreter lock): column
    blocks of the column-major DEM and output files and pulse blocks of the
    raw file are contiguous byte ranges, read straight into pinned buffers
    and written from them, with no page faults on memory maps."""

    CHUNK = 8 << 20

    def __init__(self, threads: int | None = None):
        from concurrent.futures import ThreadPoolExecutor
        self.threads = threads or min(16, os.cpu_count() or 1)
        self.pool = ThreadPoolExecutor(self.threads)
        self.fds: dict[str, int] = {}

    def fd(self, path, write: bool = False) -> int:
        key = f"{'w' if write else 'r'}:{path}"
        if key not in self.fds:
            self.fds[key] = os.open(path, os.O_RDWR if write else os.O_RDONLY)
        return self.fds[key]

    def _split(self, fn, fd, buf, pos):
        mv = memoryview(buf).cast("B")
        n = len(mv)
        step = max(self.CHUNK, -(-n // self.threads))
        futs = [self.pool.submit(fn, fd, mv[o:o + step], pos + o) for o in range(0, n, step)]
        for f in futs:
            f.result()

    def read(self, path, buf: np.ndarray, pos: int) -> None:
        self._split(_pread_full, self.fd(path), buf, pos)

    def write(self, path, buf: np.ndarray, pos: int) -> None:
        self._split(_pwrite_full, self.fd(path, write=True), buf, pos)

    def close(self) -> None:
        for fd in self.fds.values():
            os.close(fd)
        self.fds.clear()
        self.pool.shutdown()


class RawStreamer:
    """Streams a column-major (Nra, Naz) complex64 array into device memory
    (pulse-major rows, even pitch) in pulse blocks through two pinned
    buffers on its own stream; ``wait_for(k, stream)`` makes ``stream`` wait
    until pulses [0, k] are resident."""

    def __init__(self, raw, device, block_pulses: int = 8192, source=None):
        """``source`` (path, FileIO): read pulse blocks from the raw file
        itself (pulse a at byte 8*nra*a) instead of through ``raw``."""
        self.raw = raw
        self.source = source
        self.nra, self.naz = int(raw.shape[0]), int(raw.shape[1])
        self.pitch = self.nra + (self.nra & 1)
        self.device = device
        self.block = int(block_pulses)
        self.dev = torch.zeros((self.naz, self.pitch, 2), dtype=torch.float32, device=device)
        self.stream = torch.cuda.Stream(device)
        self.pinned = [torch.empty((self.block, self.nra), dtype=torch.complex64,
                                   pin_memory=True) for _ in range(2)]
        self.copied = [None, None]          # events: pinned buffer i free again
        self.done_upto = -1                  # last pulse enqueued
        self.events: list[tuple[int, torch.cuda.Event]] = []
        self.host_s = 0.0                    # host time filling the pinned buffers

    def _flat(self, a0: int, a1: int) -> np.ndarray:
        # pulses a0..a1-1 as a (pulses, nra) C-order view of the F-order array
        return np.asarray(self.raw[:, a0:a1]).T

    def pump(self, upto: int) -> None:
        """Enqueue uploads until pulse ``upto`` (inclusive) is covered."""
        while self.done_upto < min(upto, self.naz - 1):
            a0 = self.done_upto + 1
            a1 = min(a0 + self.block, self.naz)
            i = (a0 // self.block) & 1
            if self.copied[i] is not None:
                self.copied[i].synchronize()             # pinned buffer reusable
            t0 = time.perf_counter()
            buf = self.pinned[i][: a1 - a0]
            if self.source is not None:
                path, fio = self.source
                fio.read(path, buf.numpy(), 8 * self.nra * a0)
            else:
                with warnings.catch_warnings():
                    # a read-only memory map: torch only reads it (multi-threaded copy)
                    warnings.simplefilter("ignore", UserWarning)
                    buf.copy_(torch.from_numpy(self._flat(a0, a1)))
            self.host_s += time.perf_counter() - t0
            with torch.cuda.stream(self.stream):
                dst = torch.view_as_complex(self.dev[a0:a1])[:, : self.nra]
                dst.copy_(buf, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self.stream)
            self.copied[i] = ev
            self.events.append((a1 - 1, ev))
            self.done_upto = a1 - 1

    def wait_for(self, k: int, stream) -> None:
        self.pump(k)
        for last, ev in self.events:
            if last >= k:
                stream.wait_event(ev)
                return


class LargeSceneFocuser:
    """Focus a large scene in DEM azimuth batches with a resumable cursor."""

    def __init__(self, out_path, cursor_path=None, batch_cols: int = 2000, tuning=None,
                 device=None, block_pulses: int = 8192, diagnostics: bool = False):
        """``diagnostics`` also writes each pixel's contributor count (int32,
        ``<out>.nvalid``) and range-bin checksum (uint64, ``<out>.checksum``),
        column-major like the image, for checks against the oracle."""
        self.out_path = Path(out_path)
        self.diagnostics = bool(diagnostics)
        self.cursor_path = Path(cursor_path) if cursor_path else Path(str(out_path) + ".cursor")
        self.batch_cols = int(batch_cols)
        self.device = torch.device(device or "cuda")
        self.tuning = resolve_tuning(tuning)
        # one prepared workspace serves every batch: its chunk tables depend
        # on the trajectory only, a tile queue (staged=2) on one batch's pixels
        if self.tuning.staged == 2:
            self.tuning.staged = 1
        self.block_pulses = block_pulses
        self.lib = _lib.load()
        self.launches = 0
        # host seconds of the last focus(): DEM column reads and uploads, raw
        # staging into pinned buffers, output writes
        self.timing = {"dem_s": 0.0, "raw_host_s": 0.0, "write_s": 0.0}

    def focus_files(self, data_dir, dim0, dim1, nra, naz, max_batches=None) -> np.memmap:
        """Focus the scene stored as the reference's .dat files in data_dir."""
        d = Path(data_dir)
        names = datfiles.scene_filenames(dim0, dim1, nra, naz)
        mm = {k: np.memmap(d / names[k], dtype=np.float64, mode="r", shape=(dim0, dim1),
                           order="F") for k in ("xxg1", "yyg1", "zzg1")}
        mm["Index"] = np.memmap(d / names["Index"], dtype=np.int32, mode="r",
                                shape=(dim0, dim1), order="F")
        mm["Mask"] = np.memmap(d / names["Mask"], dtype=np.uint8, mode="r",
                               shape=(dim0, dim1), order="F")
        mm["Sint"] = np.memmap(d / names["Sint"], dtype=np.int32, mode="r",
                               shape=(dim0, dim1), order="F")
        traj = {k: datfiles.read_dat(d / names[k], np.float64) for k in ("wgsx", "wgsy", "wgsz")}
        n_ra, n_az = datfiles.validate_raw_dims(d / names["RawData"], nra, naz)
        raw = datfiles.open_raw_memmap(d / names["RawData"], n_ra, n_az)
        raw, wx, wy, wz = datfiles.reconcile_trajectory(raw, traj["wgsx"], traj["wgsy"],
                                                        traj["wgsz"])
        scal = {k: float(np.fromfile(d / n, dtype=np.float64)[0])
                for k, n in datfiles.SCALAR_NAMES.items()}
        files = {k: d / names[k] for k in ("xxg1", "yyg1", "zzg1", "Mask", "Index", "Sint",
                                             "RawData")}
        return self.focus(mm["xxg1"], mm["yyg1"], mm["zzg1"], mm["Mask"], mm["Index"], wx, wy,
                          wz, raw, scal["NearRange"], scal["DeltaRange"], scal["Lambda"],
                          mm["Sint"], max_batches=max_batches, files=files)

    def focus(self, xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data, near_range,
              dra, lambda_val, Sint, max_batches=None, files=None) -> np.memmap:
        """Same 13 arguments as FocalizzatoreBpPx (arrays may be memory maps).

        Returns the output memory map (complex128, (dim0, dim1), column-major).
        ``max_batches`` stops after that many batches (the cursor keeps the
        position, a later call resumes).  ``files`` (argument name -> path
        of its column-major .dat file, as focus_files passes it): the DEM
        column blocks and raw pulse blocks are read from those files by
        positional reads into pinned buffers, and the image is written the
        same way; otherwise the arrays are read where they lie.
        """
        dim0, dim1 = (int(v) for v in xxg1.shape)
        nra, naz = (int(v) for v in Raw_Data.shape)
        if len(wgsx) < naz:
            raise ValueError("trajectory shorter than Raw_Data's pulses")
        nb = (dim1 + self.batch_cols - 1) // self.batch_cols
        cur = Cursor(dim0, dim1, nra, naz, self.batch_cols)
        old = Cursor.load(self.cursor_path)
        resume = old is not None and old.matches(cur) and self.out_path.exists()
        if resume:
            cur.next_batch = old.next_batch
        mode = "r+" if resume else "w+"
        out = np.memmap(self.out_path, dtype=np.complex128, mode=mode, shape=(dim0, dim1),
                        order="F")
        self.nvalid = self.checksum = None
        if self.diagnostics:
            self.nvalid = np.memmap(str(self.out_path) + ".nvalid", dtype=np.int32, mode=mode,
                                    shape=(dim0, dim1), order="F")
            self.checksum = np.memmap(str(self.out_path) + ".checksum", dtype=np.uint64,
                                      mode=mode, shape=(dim0, dim1), order="F")
        if cur.next_batch >= nb:
            return out
        dev = self.device
        compute = torch.cuda.Stream(dev)
        side = torch.cuda.Stream(dev)
        fio = FileIO() if files else None
        self._fio = fio
        streamer = RawStreamer(Raw_Data, dev, self.block_pulses,
                               source=(files["RawData"], fio) if files else None)
        traj = [torch.as_tensor(np.ascontiguousarray(w[:naz], dtype=np.float64)).to(dev)
                for w in (wgsx, wgsy, wgsz)]
        tb = C.byref(self.tuning)
        ws = None
        from concurrent.futures import ThreadPoolExecutor
        writer = ThreadPoolExecutor(1)
        pending = None                   # the previous batch's write
        done = 0
        for b in range(cur.next_batch, nb):
            if max_batches is not None and done >= max_batches:
                break
            c0, c1 = b * self.batch_cols, min(dim1, (b + 1) * self.batch_cols)
            t0 = time.perf_counter()
            grid = (("x", xxg1, np.float64), ("y", yyg1, np.float64), ("z", zzg1, np.float64),
                    ("m", mask, np.uint8), ("i", index, np.int32), ("s", Sint, np.int32))
            fkey = {"x": "xxg1", "y": "yyg1", "z": "zzg1", "m": "Mask", "i": "Index",
                    "s": "Sint"}
            # the batch's columns go up on the side stream, where the pulse
            # window its apertures need is computed and read back: the host
            # then waits for that upload only, not for the batch before
            with torch.cuda.stream(side):
                if files:
                    # column block [c0, c1) = one contiguous byte range of each file
                    dcol = {}
                    for k, _, dt in grid:
                        es = np.dtype(dt).itemsize
                        pin = torch.empty(dim0 * (c1 - c0) * es, dtype=torch.uint8,
                                          pin_memory=True)
                        fio.read(files[fkey[k]], pin.numpy(), c0 * dim0 * es)
                        dcol[k] = pin.view(getattr(torch, np.dtype(dt).name)).to(
                            dev, non_blocking=True)
                else:
                    dcol = {k: flatten_f(np.asarray(a[:, c0:c1]), dt, dev) for k, a, dt in grid}
                rng_host = pulse_range_tensor(dcol["i"], dcol["s"], dcol["m"], naz).to(
                    "cpu", non_blocking=True)
                got = torch.cuda.Event()
                got.record(side)
            for t in dcol.values():
                t.record_stream(compute)
            compute.wait_stream(side)
            got.synchronize()
            lo, hi = int(rng_host[0]), int(rng_host[1])
            if lo > hi:
                lo, hi = 0, -1
            with torch.cuda.stream(compute):
                sc = DeviceScene(
                    dim0=dim0, dim1=c1 - c0, x=dcol["x"], y=dcol["y"], z=dcol["z"],
                    mask=dcol["m"], index=dcol["i"], sint=dcol["s"],
                    tx=traj[0], ty=traj[1], tz=traj[2], raw=streamer.dev, nra=nra, naz=naz,
                    pitch=streamer.pitch, near_range=float(near_range), delta_range=float(dra),
                    lambda_=float(lambda_val))
            self.timing["dem_s"] += time.perf_counter() - t0
            streamer.wait_for(max(hi, 0), compute)
            with torch.cuda.stream(compute):
                sp = compute.cuda_stream
                if ws is None:
                    need = _lib.check(int(self.lib.sarbp_mixed_workspace_size(
                        C.byref(sc.struct()), tb)))
                    ws = torch.empty(need, dtype=torch.uint8, device=dev)
                    _lib.check(self.lib.sarbp_mixed_prepare(C.byref(sc.struct()), tb,
                                                            ws.data_ptr(), need, sp))
                    self.launches += 1
                img = torch.empty((sc.npix, 2), dtype=torch.float64, device=dev)
                diag = None
                if self.diagnostics:
                    diag = (torch.empty(sc.npix, dtype=torch.int32, device=dev),
                            torch.empty(sc.npix, dtype=torch.int64, device=dev))
                _lib.check(self.lib.sarbp_focus_mixed_prepared(
                    C.byref(sc.struct()), tb, img.data_ptr(),
                    diag[0].data_ptr() if diag else None, diag[1].data_ptr() if diag else None,
                    None, ws.data_ptr(), ws.numel(), sp))
                self.launches += 1
                host = torch.empty((sc.npix, 2), dtype=torch.float64, pin_memory=True)
                host.copy_(img, non_blocking=True)
                if diag:
                    host = (host, diag[0].to("cpu", non_blocking=True),
                            diag[1].to("cpu", non_blocking=True))
                ev = torch.cuda.Event()
                ev.record(compute)
            # the image goes to its file on the writer thread (one batch in
            # flight: the cursor advances in batch order)
            if pending is not None:
                pending.result()
            pending = writer.submit(self._write, out, cur, b, c0, c1, host, ev)
            done += 1
            streamer.pump(hi + self.block_pulses)          # keep the copy engine busy
        if pending is not None:
            pending.result()
        writer.shutdown()
        torch.cuda.synchronize(dev)
        self.timing["raw_host_s"] = streamer.host_s
        if fio is not None:
            fio.close()
        self._fio = None
        return out

    def _write(self, out, cur: Cursor, b, c0, c1, host, ev):
        ev.synchronize()
        t0 = time.perf_counter()
        diag = None
        if isinstance(host, tuple):
            host, *diag = host
        shape = (out.shape[0], c1 - c0)
        dim0 = out.shape[0]
        fio = getattr(self, "_fio", None)
        if fio is not None:
            # the block's column-major pixels are one byte range of each file
            # (the memory maps share the page cache with these writes)
            fio.write(self.out_path, host.numpy(), c0 * dim0 * 16)
            if diag:
                fio.write(str(self.out_path) + ".nvalid", diag[0].numpy(), c0 * dim0 * 4)
                fio.write(str(self.out_path) + ".checksum", diag[1].numpy(), c0 * dim0 * 8)
        else:
            flat = host.numpy().view(np.complex128).reshape(-1)
            out[:, c0:c1] = np.reshape(flat, shape, order="F")
            out.flush()
            if diag:
                self.nvalid[:, c0:c1] = np.reshape(diag[0].numpy(), shape, order="F")
                self.checksum[:, c0:c1] = np.reshape(diag[1].numpy().view(np.uint64), shape,
                                                     order="F")
                self.nvalid.flush()
                self.checksum.flush()
        self.timing["write_s"] += time.perf_counter() - t0
        cur.next_batch = b + 1
        cur.save(self.cursor_path)
