"""Many scenes of uneven size focused in one persistent launch.

The reference focuses one scene per call and, inside a call, launches one
kernel per pixel batch with host copies in between (gpu_small_dataset.py:
285-339, main_gpu.py:415-586).  Here every pixel tile of every scene is an
item of one device work queue, ordered by decreasing estimated cost (the sum
of the tile's kept aperture lengths, so the longest items start first), and
a persistent grid of CTAs drains it in a single launch.  The whole step --
per-scene chunk tables, queue reset, persistent kernel -- can be captured
once in a CUDA graph and replayed.

``Autotuner`` picks the pixel-tile shape (and therefore the window the TMA
stages per pulse chunk) for a batch by timing the candidates on the batch
itself, and caches the choice per batch signature.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import torch

from . import _lib
from .focuser import resolve_tuning
from .scene import DeviceScene

# (tile0, tile1, window, chunk) variants of the staged kernel the autotuner times
STAGED_TILINGS = ((16, 16, 208, 64), (16, 16, 208, 128), (16, 16, 160, 128), (16, 8, 128, 64),
                  (16, 8, 128, 128), (32, 8, 128, 64))


ORDERS = ("cost", "bucket", "natural")


def item_order(cost: torch.Tensor, how: str = "cost", buckets: int = 8) -> torch.Tensor:
    """Processing order of the (scene, tile) items listed scene by scene in
    natural tile order: "cost" by decreasing estimated cost (the longest
    items start first, so no wave ends half empty); "bucket" by decreasing
    cost class (``buckets`` classes of equal width up to the largest cost),
    natural order within a class, so neighbouring tiles, whose raw windows
    overlap, still run close together in time and share L2; "natural" as
    listed."""
    n = cost.numel()
    if how == "natural" or n == 0:
        return torch.arange(n, device=cost.device)
    if how == "cost":
        return torch.argsort(cost, descending=True, stable=True)
    top = max(int(cost.max().item()), 1)
    cls = torch.clamp(cost * buckets // (top + 1), max=buckets - 1)
    return torch.argsort(-cls, stable=True)


def staged_tuning(tile0: int = 16, tile1: int = 16, window: int = 208, chunk: int = 64,
                  stage: int = 32) -> _lib.Tuning:
    return resolve_tuning({"chunk": chunk, "tile0": tile0, "tile1": tile1, "staged": 1,
                           "window": window, "stage": stage})


def _stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


@dataclass
class _SceneSlot:
    scene: DeviceScene
    ws: torch.Tensor
    out: torch.Tensor
    nvalid: torch.Tensor | None
    checksum: torch.Tensor | None
    ntiles: int


class BatchFocuser:
    """Focus a list of device-resident scenes in one persistent launch.

    ``run()`` enqueues the whole step (chunk tables of every scene, queue
    reset, persistent kernel) on the current stream; with ``graph=True`` the
    step is captured once in a CUDA graph and ``run()`` replays it.
    Outputs stay on the device: ``images()`` returns one complex128 (dim0,
    dim1) tensor per scene (column-major pixel order as the reference).
    """

    def __init__(self, scenes: list[DeviceScene], tuning=None, diagnostics: bool = False,
                 graph: bool = True, order: str = "cost"):
        if not scenes:
            raise ValueError("BatchFocuser needs at least one scene")
        self.lib = _lib.load()
        self.device = scenes[0].device
        self.tuning = staged_tuning() if tuning is None else resolve_tuning(tuning)
        if not self.tuning.staged or self.tuning.chunk not in (32, 64, 128):
            raise ValueError("the batch path runs the staged kernel (staged=1, chunk 32/64/128)")
        # the batch has its own (scene, tile) queue: no per-scene tile queue
        self.tuning.staged = 1
        self.diagnostics = diagnostics
        if order not in ORDERS:
            raise ValueError(f"order must be one of {ORDERS}")
        self.order = order
        self.counters = (torch.zeros(_lib.NUM_COUNTERS, dtype=torch.int64, device=self.device)
                         if diagnostics else None)
        tb = C.byref(self.tuning)
        self.slots: list[_SceneSlot] = []
        for sc in scenes:
            if sc.device != self.device:
                raise ValueError("all scenes of a batch must be on one device")
            s = C.byref(sc.struct())
            need = _lib.check(int(self.lib.sarbp_mixed_workspace_size(s, tb)))
            nt = _lib.check(int(self.lib.sarbp_tile_count(s, tb)))
            self.slots.append(_SceneSlot(
                scene=sc, ws=torch.empty(need, dtype=torch.uint8, device=self.device),
                out=torch.zeros((sc.npix, 2), dtype=torch.float64, device=self.device),
                nvalid=(torch.zeros(sc.npix, dtype=torch.int32, device=self.device)
                        if diagnostics else None),
                checksum=(torch.zeros(sc.npix, dtype=torch.int64, device=self.device)
                          if diagnostics else None),
                ntiles=nt))
        self.n_items = sum(sl.ntiles for sl in self.slots)
        self.bws_bytes = _lib.check(int(self.lib.sarbp_batch_workspace_size(len(self.slots),
                                                                            self.n_items)))
        self.bws = torch.empty(self.bws_bytes, dtype=torch.uint8, device=self.device)
        self._prepare_tables()
        self._describe()
        self._plan()
        self.graph = None
        if graph:
            self._capture()

    # -- set-up ------------------------------------------------------------

    def _prepare_tables(self):
        tb = C.byref(self.tuning)
        sp = _stream_ptr(self.device)
        for sl in self.slots:
            _lib.check(self.lib.sarbp_mixed_prepare(C.byref(sl.scene.struct()), tb,
                                                    sl.ws.data_ptr(), sl.ws.numel(), sp))

    def _describe(self):
        tb = C.byref(self.tuning)
        sp = _stream_ptr(self.device)
        for i, sl in enumerate(self.slots):
            _lib.check(self.lib.sarbp_batch_set_scene(
                self.bws.data_ptr(), self.bws_bytes, len(self.slots), i,
                C.byref(sl.scene.struct()), tb, sl.ws.data_ptr(), sl.ws.numel(),
                sl.out.data_ptr(), sl.nvalid.data_ptr() if sl.nvalid is not None else None,
                sl.checksum.data_ptr() if sl.checksum is not None else None, sp))

    def _plan(self):
        """Queue of (slot, tile) items in decreasing estimated cost."""
        tb = C.byref(self.tuning)
        sp = _stream_ptr(self.device)
        costs, slot_ids, tile_ids = [], [], []
        for i, sl in enumerate(self.slots):
            c = torch.empty(sl.ntiles, dtype=torch.int64, device=self.device)
            _lib.check(self.lib.sarbp_tile_costs(C.byref(sl.scene.struct()), tb, c.data_ptr(),
                                                 sp))
            costs.append(c)
            slot_ids.append(torch.full((sl.ntiles,), i, dtype=torch.int32, device=self.device))
            tile_ids.append(torch.arange(sl.ntiles, dtype=torch.int32, device=self.device))
        cost = torch.cat(costs)
        order = item_order(cost, self.order)
        items = torch.stack([torch.cat(slot_ids)[order], torch.cat(tile_ids)[order]], dim=1)
        self.items = items.to(torch.int32).cpu().contiguous()
        self.total_cost = int(cost.sum().item())
        _lib.check(self.lib.sarbp_batch_set_items(self.bws.data_ptr(), self.bws_bytes,
                                                  len(self.slots),
                                                  self.items.data_ptr(), self.n_items, sp))

    def _launch(self):
        tb = C.byref(self.tuning)
        sp = _stream_ptr(self.device)
        for sl in self.slots:
            _lib.check(self.lib.sarbp_mixed_prepare(C.byref(sl.scene.struct()), tb,
                                                    sl.ws.data_ptr(), sl.ws.numel(), sp))
        _lib.check(self.lib.sarbp_batch_focus(
            self.bws.data_ptr(), self.bws_bytes, len(self.slots), tb, self.n_items,
            1 if self.diagnostics else 0,
            self.counters.data_ptr() if self.counters is not None else None, sp))

    def _capture(self):
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            self._launch()                      # warm-up outside the capture
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch()

    # -- use ---------------------------------------------------------------

    def run(self):
        """Enqueue one focusing step of the whole batch on the current stream."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._launch()

    def images(self) -> list[torch.Tensor]:
        return [torch.view_as_complex(sl.out).reshape(sl.scene.dim1, sl.scene.dim0).t()
                for sl in self.slots]

    def nominal_pixel_pulses(self) -> int:
        return sum(sl.scene.nominal_pixel_pulses() for sl in self.slots)

    def launches_per_step(self) -> int:
        return len(self.slots) + 1


class Autotuner:
    """Pick the fastest staged tiling for a set of scenes, by timing on it."""

    def __init__(self, candidates=STAGED_TILINGS, repeats: int = 3):
        self.candidates = candidates
        self.repeats = repeats
        self.cache: dict[tuple, tuple] = {}
        self.timings: dict[tuple, dict] = {}

    @staticmethod
    def signature(scenes: list[DeviceScene]) -> tuple:
        pix = sum(s.npix for s in scenes)
        naz = sum(s.naz for s in scenes) / len(scenes)
        return (len(scenes), int(math.log2(max(pix, 1))), int(math.log2(max(naz, 1))),
                int(sum(s.nra for s in scenes) / len(scenes)) // 256)

    def pick(self, scenes: list[DeviceScene]) -> _lib.Tuning:
        key = self.signature(scenes)
        if key not in self.cache:
            best, times = None, {}
            for cand in self.candidates:
                bf = BatchFocuser(scenes, staged_tuning(*cand), graph=False)
                bf.run()
                torch.cuda.synchronize(bf.device)
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(self.repeats):
                    bf.run()
                b.record()
                torch.cuda.synchronize(bf.device)
                ms = a.elapsed_time(b) / self.repeats
                times["{}x{}/{}/c{}".format(*cand)] = ms
                if best is None or ms < best[0]:
                    best = (ms, cand)
                del bf
            self.cache[key] = best[1]
            self.timings[key] = times
        return staged_tuning(*self.cache[key])


def time_steps(fn, steps: int, device) -> float:
    """Mean milliseconds per call of ``fn`` over ``steps`` calls (CUDA events)."""
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize(device)
    return a.elapsed_time(b) / steps


def wall(fn) -> float:
    t0 = time.perf_counter()
    fn()
    return time.perf_counter() - t0
