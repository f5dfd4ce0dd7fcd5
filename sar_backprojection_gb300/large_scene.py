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


def batch_pulse_range(index_cols: np.ndarray, sint_cols: np.ndarray, mask_cols: np.ndarray,
                      naz: int) -> tuple[int, int]:
    """[lo, hi] of the pulses the kept apertures of a DEM batch reach, or (0, -1)."""
    s = np.asarray(sint_cols, dtype=np.int64).reshape(-1)
    idx = np.asarray(index_cols, dtype=np.int64).reshape(-1)
    m = np.asarray(mask_cols).astype(np.uint8).reshape(-1)
    ok = (m == 1) & (s != -9999)
    half = np.where(s >= 0, (s + 1) // 2, -((-s) // 2))
    jj = half * 2 + 1
    off = (np.abs(s) + 1) // 2
    ok &= jj > 0
    if not ok.any():
        return 0, -1
    lo = np.maximum(idx[ok] - off[ok], 1)
    hi = np.minimum(idx[ok] - off[ok] + jj[ok] - 1, naz - 2)
    keep = lo <= hi
    if not keep.any():
        return 0, -1
    return int(lo[keep].min()), int(hi[keep].max())


class RawStreamer:
    """Streams a column-major (Nra, Naz) complex64 array into device memory
    (pulse-major rows, even pitch) in pulse blocks through two pinned
    buffers on its own stream; ``wait_for(k, stream)`` makes ``stream`` wait
    until pulses [0, k] are resident."""

    def __init__(self, raw, device, block_pulses: int = 8192):
        self.raw = raw
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
            buf = self.pinned[i][: a1 - a0]
            buf.numpy()[:] = self._flat(a0, a1)
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
                 device=None, block_pulses: int = 8192):
        self.out_path = Path(out_path)
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
        return self.focus(mm["xxg1"], mm["yyg1"], mm["zzg1"], mm["Mask"], mm["Index"], wx, wy,
                          wz, raw, scal["NearRange"], scal["DeltaRange"], scal["Lambda"],
                          mm["Sint"], max_batches=max_batches)

    def focus(self, xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data, near_range,
              dra, lambda_val, Sint, max_batches=None) -> np.memmap:
        """Same 13 arguments as FocalizzatoreBpPx (arrays may be memory maps).

        Returns the output memory map (complex128, (dim0, dim1), column-major).
        ``max_batches`` stops after that many batches (the cursor keeps the
        position, a later call resumes).
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
        out = np.memmap(self.out_path, dtype=np.complex128, mode="r+" if resume else "w+",
                        shape=(dim0, dim1), order="F")
        if cur.next_batch >= nb:
            return out
        dev = self.device
        compute = torch.cuda.Stream(dev)
        streamer = RawStreamer(Raw_Data, dev, self.block_pulses)
        traj = [torch.as_tensor(np.ascontiguousarray(w[:naz], dtype=np.float64)).to(dev)
                for w in (wgsx, wgsy, wgsz)]
        tb = C.byref(self.tuning)
        ws = None
        pending = None                   # (batch index, host buffer, event)
        done = 0
        for b in range(cur.next_batch, nb):
            if max_batches is not None and done >= max_batches:
                break
            c0, c1 = b * self.batch_cols, min(dim1, (b + 1) * self.batch_cols)
            cols = {k: np.asarray(a[:, c0:c1]) for k, a in
                    (("x", xxg1), ("y", yyg1), ("z", zzg1), ("m", mask), ("i", index),
                     ("s", Sint))}
            lo, hi = batch_pulse_range(cols["i"], cols["s"], cols["m"], naz)
            with torch.cuda.stream(compute):
                sc = DeviceScene(
                    dim0=dim0, dim1=c1 - c0,
                    x=flatten_f(cols["x"], np.float64, dev), y=flatten_f(cols["y"], np.float64, dev),
                    z=flatten_f(cols["z"], np.float64, dev),
                    mask=flatten_f(cols["m"], np.uint8, dev),
                    index=flatten_f(cols["i"], np.int32, dev),
                    sint=flatten_f(cols["s"], np.int32, dev),
                    tx=traj[0], ty=traj[1], tz=traj[2], raw=streamer.dev, nra=nra, naz=naz,
                    pitch=streamer.pitch, near_range=float(near_range), delta_range=float(dra),
                    lambda_=float(lambda_val))
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
                _lib.check(self.lib.sarbp_focus_mixed_prepared(
                    C.byref(sc.struct()), tb, img.data_ptr(), None, None, None, ws.data_ptr(),
                    ws.numel(), sp))
                self.launches += 1
                host = torch.empty((sc.npix, 2), dtype=torch.float64, pin_memory=True)
                host.copy_(img, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(compute)
            if pending is not None:
                self._write(out, cur, *pending)
            pending = (b, c0, c1, host, ev)
            done += 1
            streamer.pump(hi + self.block_pulses)          # keep the copy engine busy
        if pending is not None:
            self._write(out, cur, *pending)
        torch.cuda.synchronize(dev)
        return out

    def _write(self, out, cur: Cursor, b, c0, c1, host, ev):
        ev.synchronize()
        flat = host.numpy().view(np.complex128).reshape(-1)
        out[:, c0:c1] = np.reshape(flat, (out.shape[0], c1 - c0), order="F")
        out.flush()
        cur.next_batch = b + 1
        cur.save(self.cursor_path)
