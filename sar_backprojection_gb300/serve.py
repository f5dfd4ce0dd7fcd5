"""Continuous-batching focusing service on one GPU.

Requests (focusing jobs of different sizes) arrive over time.  The engine

* admits a waiting job as soon as a scene slot and enough of the HBM budget
  are free (at most ``ADMIT_PER_PASS`` per pass of the loop, so waves keep
  launching during a burst of arrivals), without waiting for the GPU: its
  small inputs, chunk tables and reachable-range-bin bound are queued on a
  setup stream of their own, the bound comes back to pinned host memory in
  stream order, and on a later pass, once the host sees it, only the range
  bins the job's apertures can reach are copied from host raw data on the
  copy stream (the job's raw data and trajectory stay resident until it
  finishes); page-locked inputs go up by SM loads (``h2d="sm"``), which
  on this hardware do not share the copy engine's occasional stalls;
* runs the device in *waves*: each wave is one launch of the persistent
  batch kernel whose work queue holds pixel tiles of every resident job (one
  whose raw copy the host has seen complete), so a job that arrives while
  others are on the GPU joins a later wave and its tiles run alongside
  theirs, and no wave ever waits for an upload; waves alternate between two
  streams and two batch workspaces, so the next wave is already on the
  device and its CTAs fill the tail of the running one;
* reads a job's image back (pinned host memory, on a read-back stream that
  no upload queues ahead of) when its last tile is done, then frees its slot
  and memory.

Latency = completion of the image's device-to-host copy minus arrival time.
Per-tile work is the same code as the single-scene kernel, so a job's image
is bit-identical whether it ran alone or in the mix.
"""
from __future__ import annotations

import ctypes as C
import gc
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .batch import staged_tuning
from .focuser import resolve_tuning
from .scene import DeviceScene, read_bound, scene_to_device

GB = 1 << 30
ADMIT_PER_PASS = 2     # admissions per pass of the serving loop


def job_bytes(dim0: int, dim1: int, nra: int, naz: int) -> int:
    """Device bytes a job holds while resident (inputs, image, workspace)."""
    npix = dim0 * dim1
    pitch = nra + (nra & 1)
    return (8 * pitch * naz + 37 * npix + 24 * naz + 16 * npix + 56 * naz + 4096)


@dataclass
class Job:
    """One focusing request: the reference's 13 positional arguments."""

    job_id: int
    args: tuple
    arrival: float = 0.0                  # seconds after the start of the run
    admitted: float | None = None
    finished: float | None = None
    image: np.ndarray | None = None
    nominal: int = 0

    @property
    def shape(self):
        return tuple(self.args[0].shape)

    def nbytes(self) -> int:
        raw = self.args[8]
        return job_bytes(self.shape[0], self.shape[1], int(raw.shape[0]), int(raw.shape[1]))

    @property
    def latency(self) -> float | None:
        return None if self.finished is None else self.finished - self.arrival


@dataclass
class _Active:
    job: Job
    slot: int
    scene: DeviceScene
    ws: torch.Tensor
    out: torch.Tensor
    host: torch.Tensor
    ntiles: int                           # tiles of the job's scene
    next_tile: int = 0                    # tiles [next_tile, ntiles) not yet launched
    staged: torch.cuda.Event | None = None     # small inputs, tables, bound, scene slot
    uploaded: torch.cuda.Event | None = None   # raw data on the device (copy issued)
    resident: bool = False                # the host has seen `uploaded` complete
    in_flight: int = 0
    done_event: torch.cuda.Event | None = None


@dataclass
class ServingReport:
    jobs: list
    wall_s: float
    waves: int
    gpu_launches: int
    peak_bytes: int
    latencies_ms: list = field(default_factory=list)
    h2d_bytes: int | None = None          # native engine: bytes uploaded / read back
    d2h_bytes: int | None = None

    def summary(self) -> dict:
        lat = np.array([j.latency for j in self.jobs if j.latency is not None]) * 1e3
        work = sum(j.nominal for j in self.jobs)
        return {"jobs": len(self.jobs), "completed": int(lat.size),
                "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
                "mean_ms": float(lat.mean()) if lat.size else None,
                "wall_s": self.wall_s, "pixel_pulses": work,
                "gpix_pulse_per_s": work / self.wall_s / 1e9 if self.wall_s > 0 else None,
                "waves": self.waves, "gpu_launches": self.gpu_launches,
                "peak_resident_gb": self.peak_bytes / GB if self.peak_bytes else None,
                "h2d_gb": self.h2d_bytes / 1e9 if self.h2d_bytes is not None else None,
                "d2h_gb": self.d2h_bytes / 1e9 if self.d2h_bytes is not None else None,
                "h2d_gb_per_s": (self.h2d_bytes / 1e9 / self.wall_s
                                 if self.h2d_bytes is not None and self.wall_s > 0 else None)}


class ServingEngine:
    """Continuous batching of focusing jobs on one device (see module doc)."""

    def __init__(self, device=None, budget_bytes: int = 150 * GB, max_slots: int = 32,
                 wave_items: int | None = None, tuning=None, policy: str = "fifo",
                 h2d: str = "sm"):
        if policy not in ("fifo", "srpt"):
            raise ValueError("policy must be 'fifo' or 'srpt'")
        if h2d not in ("copy", "sm"):
            raise ValueError("h2d must be 'copy' or 'sm'")
        self.device = torch.device(device or "cuda")
        self.lib = _lib.load()
        self.tuning = staged_tuning() if tuning is None else resolve_tuning(tuning)
        self.budget = int(budget_bytes)
        self.max_slots = int(max_slots)
        props = torch.cuda.get_device_properties(self.device)
        self.wave_items = int(wave_items or 3 * 2 * props.multi_processor_count)
        self.policy = policy
        # page-locked job inputs go up by SM loads ("sm", sarbp_*_sm): the
        # copy engine's host-to-device transfers stall now and then on this
        # hardware and every job queued behind a stall waits; "copy" uses it
        self.h2d = h2d
        self.compute = [torch.cuda.Stream(self.device), torch.cuda.Stream(self.device)]
        self.setup = torch.cuda.Stream(self.device)      # small inputs, tables, bound
        self.copy = torch.cuda.Stream(self.device)       # raw range bins
        self.readback = torch.cuda.Stream(self.device)   # images to host memory
        nb = _lib.check(int(self.lib.sarbp_batch_workspace_size(self.max_slots,
                                                                self.wave_items)))
        self.bws_bytes = nb
        self.bws = [torch.empty(nb, dtype=torch.uint8, device=self.device) for _ in range(2)]
        self.free_slots = list(range(self.max_slots))
        # per slot: the reachable-bin bound of the job in it (pinned, written
        # by the device in stream order)
        self.bounds = torch.empty((self.max_slots, 2), dtype=torch.int32, pin_memory=True)
        self.used = 0
        self.peak = 0

    # -- per job -----------------------------------------------------------

    def _admit(self, job: Job, now: float) -> _Active:
        slot = self.free_slots.pop(0)
        tb = C.byref(self.tuning)
        with torch.cuda.stream(self.setup):
            # small inputs, chunk tables (prepared with the serving tuning),
            # the reachable-bin bound into this slot's pinned pair and the
            # batch scene slot, all queued on the setup stream: nothing here
            # waits for the GPU
            scene = scene_to_device(*job.args, device=self.device, raw_bins="deferred",
                                    tuning=self.tuning, bound_host=self.bounds[slot],
                                    h2d=self.h2d)
            ws_bytes = _lib.check(int(self.lib.sarbp_mixed_workspace_size(
                C.byref(scene.struct()), tb)))
            out = torch.empty((scene.npix, 2), dtype=torch.float64, device=self.device)
            sp = self.setup.cuda_stream
            if scene.workspace is not None and scene.workspace.numel() >= ws_bytes:
                ws = scene.workspace            # prepared with this tuning on the way
            else:
                ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.device)
                _lib.check(self.lib.sarbp_mixed_prepare(C.byref(scene.struct()), tb,
                                                        ws.data_ptr(), ws_bytes, sp))
            nt = _lib.check(int(self.lib.sarbp_tile_count(C.byref(scene.struct()), tb)))
            for b in self.bws:
                _lib.check(self.lib.sarbp_batch_set_scene(
                    b.data_ptr(), self.bws_bytes, self.max_slots, slot, C.byref(scene.struct()),
                    tb, ws.data_ptr(), ws_bytes, out.data_ptr(), None, None, sp))
        staged = torch.cuda.Event()
        staged.record(self.setup)
        job.admitted = now
        host = torch.empty((scene.npix, 2), dtype=torch.float64, pin_memory=True)
        self.used += job.nbytes()
        self.peak = max(self.peak, self.used)
        return _Active(job=job, slot=slot, scene=scene, ws=ws, out=out, host=host,
                       ntiles=nt, staged=staged)

    def _start_upload(self, a: _Active) -> None:
        """The job's setup has completed: copy its reachable raw bins (host raw
        data in the reference's layout), queued behind earlier jobs' copies."""
        scene = a.scene
        self.copy.wait_event(a.staged)
        if scene.host_rows is not None:
            lo, hi = read_bound(scene)
            if hi >= lo:
                n = hi - lo + 1
                upload = (self.lib.sarbp_upload_raw_bins_sm
                          if self.h2d == "sm" and scene.host_rows.is_pinned()
                          else self.lib.sarbp_upload_raw_bins)
                _lib.check(upload(scene.raw.data_ptr(), scene.pitch, scene.host_rows.data_ptr(),
                                  scene.nra, lo, n, scene.naz, self.copy.cuda_stream))
                scene.h2d_bytes += n * scene.naz * 8
        a.uploaded = torch.cuda.Event()
        a.uploaded.record(self.copy)

    def _retire(self, a: _Active, now: float):
        j = a.job
        flat = a.host.numpy().view(np.complex128).reshape(-1)
        j.image = np.reshape(flat, (a.scene.dim0, a.scene.dim1), order="F")
        j.finished = now
        self.used -= j.nbytes()
        self.free_slots.append(a.slot)

    # -- waves -------------------------------------------------------------

    def _build_wave(self, active: list[_Active]) -> list[tuple[_Active, int, int]]:
        """Up to ``wave_items`` tiles as (job, first, end) tile ranges, one per
        job: FIFO takes the oldest jobs' tiles first, SRPT the jobs with the
        fewest tiles left."""
        cand = [a for a in active if a.next_tile < a.ntiles]
        if self.policy == "srpt":
            cand.sort(key=lambda a: a.ntiles - a.next_tile)
        else:
            cand.sort(key=lambda a: a.job.arrival)
        wave = []
        room = self.wave_items
        for a in cand:
            if room == 0:
                break
            take = min(room, a.ntiles - a.next_tile)
            wave.append((a, a.next_tile, a.next_tile + take))
            a.next_tile += take
            room -= take
        return wave

    def _launch_wave(self, wave, turn: int) -> torch.cuda.Event:
        n = sum(t1 - t0 for _, t0, t1 in wave)
        items = np.empty((n, 2), dtype=np.int32)        # (slot, tile) work items
        k = 0
        for a, t0, t1 in wave:
            items[k:k + t1 - t0, 0] = a.slot
            items[k:k + t1 - t0, 1] = np.arange(t0, t1, dtype=np.int32)
            k += t1 - t0
            a.in_flight += 1
        stream, bws = self.compute[turn], self.bws[turn]
        with torch.cuda.stream(stream):
            sp = stream.cuda_stream
            _lib.check(self.lib.sarbp_batch_set_items(bws.data_ptr(), self.bws_bytes,
                                                      self.max_slots,
                                                      items.ctypes.data_as(C.c_void_p),
                                                      n, sp))
            _lib.check(self.lib.sarbp_batch_focus(bws.data_ptr(), self.bws_bytes,
                                                  self.max_slots, C.byref(self.tuning),
                                                  n, 0, None, sp))
        ev = torch.cuda.Event()
        ev.record(stream)
        return ev

    # -- the loop ----------------------------------------------------------

    def run(self, jobs: list[Job], clock=time.perf_counter, idle_sleep: float = 5e-5,
            timeout_s: float = 600.0) -> ServingReport:
        # the loop runs with the cyclic garbage collector paused: its objects
        # are freed by reference counting, and a full collection of a large
        # interpreter heap stalls the loop (and every job in flight) for tens
        # of milliseconds
        gc_was_enabled = gc.isenabled()
        gc.disable()
        try:
            return self._run(jobs, clock, idle_sleep, timeout_s)
        finally:
            if gc_was_enabled:
                gc.enable()

    def _run(self, jobs, clock, idle_sleep, timeout_s) -> ServingReport:
        arrivals = sorted(jobs, key=lambda j: j.arrival)
        pending: deque = deque()
        active: list[_Active] = []
        readbacks: list = []             # (event, active)
        waves_in_flight: deque = deque()  # (event, wave, ws index)
        nxt = 0
        nwaves = 0
        launches = 0
        ws_turn = 0
        t0 = clock()
        while True:
            now = clock() - t0
            if now > timeout_s:
                raise TimeoutError(f"serving run exceeded {timeout_s} s")
            while nxt < len(arrivals) and arrivals[nxt].arrival <= now:
                pending.append(arrivals[nxt])
                nxt += 1
            progress = False
            # admission: FIFO, by slots and HBM budget, a few per pass
            admitted = 0
            while (pending and admitted < ADMIT_PER_PASS and self.free_slots
                   and self.used + pending[0].nbytes() <= self.budget):
                active.append(self._admit(pending.popleft(), now))
                admitted += 1
                launches += 4            # chunk tables, bound (3); uploads are copies
                progress = True
            # jobs whose setup has completed get their raw copy; jobs whose
            # raw copy has landed may join waves
            for a in active:
                if a.uploaded is None:
                    if a.staged.query():
                        self._start_upload(a)
                        progress = True
                elif not a.resident and a.uploaded.query():
                    a.resident = True
                    progress = True
            if pending and not active and not self.free_slots:
                raise RuntimeError("no scene slot free and nothing running")
            if pending and not active and self.used + pending[0].nbytes() > self.budget:
                raise RuntimeError(f"job {pending[0].job_id} needs more than the HBM budget")
            # completed waves
            while waves_in_flight and waves_in_flight[0][0].query():
                _, wave, _ = waves_in_flight.popleft()
                progress = True
                for a, _t0, _t1 in wave:          # each job once per wave
                    a.in_flight -= 1
                    if a.next_tile >= a.ntiles and a.in_flight == 0 and a.done_event is None:
                        # every wave with this job's tiles has completed: read back
                        with torch.cuda.stream(self.readback):
                            a.host.copy_(a.out, non_blocking=True)
                            ev = torch.cuda.Event()
                            ev.record(self.readback)
                        a.done_event = ev
                        readbacks.append(a)
            # keep two waves queued on the device
            while len(waves_in_flight) < 2:
                wave = self._build_wave([a for a in active if a.resident])
                if not wave:
                    break
                turn = ws_turn
                ws_turn ^= 1
                ev = self._launch_wave(wave, turn)
                waves_in_flight.append((ev, wave, turn))
                nwaves += 1
                launches += 1
                progress = True
            # finished read-backs
            still = []
            for a in readbacks:
                if a.done_event.query():
                    self._retire(a, clock() - t0)
                    active.remove(a)
                    progress = True
                else:
                    still.append(a)
            readbacks = still
            if nxt >= len(arrivals) and not pending and not active:
                break
            if idle_sleep and not progress:
                time.sleep(idle_sleep)
        torch.cuda.synchronize(self.device)
        wall = clock() - t0
        for j in jobs:                   # accounting, outside the timed loop
            if not j.nominal:
                j.nominal = _nominal(j.args)
        return ServingReport(jobs=jobs, wall_s=wall, waves=nwaves,
                             gpu_launches=launches, peak_bytes=self.peak)


def _nominal(args) -> int:
    """Nominal pixel-pulses of a job from its host Mask and Sint arguments."""
    m = np.asarray(args[3]).astype(np.uint8).reshape(-1)
    s = np.asarray(args[12]).astype(np.int64).reshape(-1)
    jj = np.where(s >= 0, (s + 1) // 2, -((-s) // 2)) * 2 + 1
    return int(np.where((m == 1) & (s != -9999) & (jj > 0), jj, 0).sum())


def poisson_arrivals(n: int, rate_per_s: float, seed: int = 0) -> np.ndarray:
    """Arrival times (s) of a Poisson process with the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, n))


def run_fp64_sequential(jobs: list[Job], device=None) -> dict:
    """Plain FP64 kernel, one job at a time in arrival order (the comparator).

    Each job is uploaded, focused and read back before the next starts; the
    service time of job k starts when both it has arrived and job k-1 is done.
    """
    from .focuser import focus
    dev = torch.device(device or "cuda")
    clock_free = 0.0
    lat = []
    work = 0
    busy = 0.0
    for j in sorted(jobs, key=lambda j: j.arrival):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sc = scene_to_device(*j.args, device=dev)
        res = focus(sc, "fp64")
        res.image.cpu()
        torch.cuda.synchronize(dev)
        svc = time.perf_counter() - t0
        start = max(j.arrival, clock_free)
        clock_free = start + svc
        lat.append(clock_free - j.arrival)
        work += sc.nominal_pixel_pulses()
        busy += svc
        del sc, res
    lat = np.array(lat) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "busy_s": busy, "pixel_pulses": work, "gpix_pulse_per_s": work / busy / 1e9}


class NativeQueue:
    """The C serving queue (sarbp_queue_*): device-resident scenes in, device
    images out; a native worker thread admits them and runs waves of the
    persistent batch kernel.  ``submit`` returns a job id; ``wait``/``poll``
    report completion (once per job)."""

    def __init__(self, tuning=None, max_slots: int = 32, wave_items: int = 0):
        self.lib = _lib.load()
        self.tuning = staged_tuning() if tuning is None else resolve_tuning(tuning)
        self._q = C.c_void_p()
        _lib.check(self.lib.sarbp_queue_create(C.byref(self._q), C.byref(self.tuning),
                                               int(max_slots), int(wave_items)))
        self._keep: dict[int, tuple] = {}

    def submit(self, scene: DeviceScene, out: torch.Tensor | None = None) -> int:
        if out is None:
            out = torch.empty((scene.npix, 2), dtype=torch.float64, device=scene.device)
        # inputs must be on the device before the worker's streams read them
        torch.cuda.current_stream(scene.device).synchronize()
        job = _lib.check(int(self.lib.sarbp_queue_submit(self._q, C.byref(scene.struct()),
                                                         out.data_ptr())))
        self._keep[job] = (scene, out)
        return job

    def poll(self, job: int) -> bool:
        done = _lib.check(int(self.lib.sarbp_queue_poll(self._q, job))) == 1
        return done

    def cancel(self, job: int) -> None:
        """Cancel a job still waiting for admission (SarbpError if it is
        already admitted); waiting on it then raises with SARBP_ECANCELED."""
        _lib.check(int(self.lib.sarbp_queue_cancel(self._q, job)))

    def wait(self, job: int) -> torch.Tensor:
        """Block until the job is done; its (npix, 2) float64 device image."""
        try:
            _lib.check(int(self.lib.sarbp_queue_wait(self._q, job)))
        finally:
            scene, out = self._keep.pop(job, (None, None))
        return out

    def close(self) -> None:
        if self._q:
            rc = int(self.lib.sarbp_queue_destroy(self._q))
            self._q = C.c_void_p()
            self._keep.clear()
            _lib.check(rc)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _host_grid(a, np_dtype):
    """(owner, pointer) of a host DEM-grid array as column-major ``np_dtype``
    data: the array itself when it already is (a NumPy F-order array or a
    CPU tensor whose transpose is contiguous, pinned memory kept), else a
    column-major copy."""
    if isinstance(a, torch.Tensor):
        tdt = getattr(torch, np.dtype(np_dtype).name)
        if a.device.type == "cpu" and a.dtype == tdt and (a.dim() != 2 or a.t().is_contiguous()):
            return a, a.data_ptr()
        a = a.detach().cpu().numpy()
    arr = np.asarray(a)
    if not (arr.dtype == np_dtype and (arr.ndim != 2 or arr.flags.f_contiguous)):
        arr = np.asfortranarray(arr.astype(np_dtype))
    return arr, arr.ctypes.data


def _host_vector(w, naz: int):
    """(owner, pointer) of a trajectory component as ``naz`` contiguous float64
    (the reference reads pulses 0 < a < Naz-1 only: a shorter trajectory of
    Naz-1 points is padded with its last point)."""
    if isinstance(w, torch.Tensor) and w.device.type == "cpu" and w.dtype == torch.float64 \
            and w.is_contiguous() and w.numel() >= naz:
        return w, w.data_ptr()
    v = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1))
    if v.size < naz:
        v = np.concatenate([v, np.full(naz - v.size, v[-1] if v.size else 0.0)])
    return v, v.ctypes.data


def host_scene(args: tuple) -> tuple:
    """The 13 focusing arguments as a host sarbp_scene (pointers into the
    caller's arrays where their layout allows, else into column-major
    copies); returns (scene struct, owners to keep alive)."""
    (xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, raw, near, dra, lam, sint) = args
    if len(tuple(raw.shape)) != 2 or len(tuple(xxg1.shape)) != 2:
        raise ValueError("Raw_Data and xxg1 must be 2D arrays")
    dim0, dim1 = (int(v) for v in xxg1.shape)
    nra, naz = (int(v) for v in raw.shape)
    keep = []
    ptr = {}
    for name, a, dt in (("dem_x", xxg1, np.float64), ("dem_y", yyg1, np.float64),
                        ("dem_z", zzg1, np.float64), ("mask", mask, np.uint8),
                        ("index", index, np.int32), ("sint", sint, np.int32)):
        if int(np.prod(tuple(a.shape))) != dim0 * dim1:
            raise ValueError(f"{name} does not match the DEM grid")
        o, p = _host_grid(a, dt)
        keep.append(o)
        ptr[name] = p
    for name, w in (("traj_x", wgsx), ("traj_y", wgsy), ("traj_z", wgsz)):
        if int(np.prod(tuple(w.shape))) < naz - 1:
            raise ValueError(f"{name} has fewer than Naz-1 points")
        o, p = _host_vector(w, naz)
        keep.append(o)
        ptr[name] = p
    o, p = _host_grid(raw, np.complex64)                  # (nra, naz) column-major rows
    keep.append(o)
    sc = _lib.Scene(dim0=dim0, dim1=dim1, nra=nra, naz=naz, raw_pitch=nra,
                    near_range=float(near), delta_range=float(dra), lambda_=float(lam),
                    raw=p, **ptr)
    return sc, keep


class NativeServingEngine:
    """Continuous batching with the whole request path in the C queue's worker
    thread (sarbp_queue_submit_host): jobs are submitted from host memory at
    their arrival times; admission by slot and reserved device memory, the
    small uploads, chunk tables, reachable-bin bound, raw upload, waves and
    the image read-back all run natively.  The Python loop only submits and
    drains completions (sarbp_queue_completed), whose times come from the
    worker (the monotonic clock).  Images are bit-identical to the
    single-scene staged kernel's."""

    def __init__(self, device=None, budget_bytes: int = 150 * GB, max_slots: int = 32,
                 wave_items: int = 0, tuning=None):
        self.device = torch.device(device or "cuda")
        self.lib = _lib.load()
        self.tuning = staged_tuning() if tuning is None else resolve_tuning(tuning)
        self.budget = int(budget_bytes)
        self._q = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.sarbp_queue_create(C.byref(self._q), C.byref(self.tuning),
                                                   int(max_slots), int(wave_items)))
            try:
                _lib.check(self.lib.sarbp_queue_reserve(self._q, self.budget))
            except Exception:
                self.lib.sarbp_queue_destroy(self._q)
                raise

    def job_bytes(self, args) -> int:
        sc, _ = host_scene(args)
        return _lib.check(int(self.lib.sarbp_queue_job_bytes(self._q, C.byref(sc))))

    def run(self, jobs: list, idle_sleep: float = 5e-5, timeout_s: float = 600.0):
        """Submit every job at its arrival time (seconds after the start),
        wait for all; returns a ServingReport (``waves``/``gpu_launches``
        are not counted by the native worker: None)."""
        prepared = []
        for j in sorted(jobs, key=lambda j: j.arrival):     # outside the timed loop
            sc, keep = host_scene(j.args)
            out = torch.empty((sc.dim0 * sc.dim1, 2), dtype=torch.float64, pin_memory=True)
            if not j.nominal:
                j.nominal = _nominal(j.args)
            prepared.append((j, sc, keep, out))

        def submit(item):
            j, sc, keep, out = item
            return self.lib.sarbp_queue_submit_host(self._q, C.byref(sc), out.data_ptr())

        def finished(item):
            j, sc, keep, out = item
            flat = out.numpy().view(np.complex128).reshape(-1)
            j.image = np.reshape(flat, (sc.dim0, sc.dim1), order="F")

        return self._drive(jobs, prepared, submit, finished, idle_sleep, timeout_s)

    def run_resident(self, jobs: list, scene_of, idle_sleep: float = 5e-5,
                     timeout_s: float = 600.0):
        """The same loop for jobs whose inputs are already resident in device
        memory (``scene_of(job)`` -> DeviceScene, sarbp_queue_submit): each
        job's image goes to a device buffer of its own; admission by slot
        and reserved memory (the chunk-table workspace is carved from it),
        waves as for host jobs.  ``job.image`` is the (npix, 2) float64
        device image."""
        prepared = []
        for j in sorted(jobs, key=lambda j: j.arrival):
            sc = scene_of(j)
            out = torch.empty((sc.npix, 2), dtype=torch.float64, device=sc.device)
            if not j.nominal:
                j.nominal = sc.nominal_pixel_pulses()
            prepared.append((j, sc, out))
        torch.cuda.synchronize(self.device)      # inputs and outputs exist before the worker

        def submit(item):
            j, sc, out = item
            return self.lib.sarbp_queue_submit(self._q, C.byref(sc.struct()), out.data_ptr())

        def finished(item):
            item[0].image = item[2]

        return self._drive(jobs, prepared, submit, finished, idle_sleep, timeout_s)

    def _drive(self, jobs, prepared, submit, finished, idle_sleep, timeout_s):
        byid = {}
        before = self.stats()
        ids = (C.c_int64 * 256)()
        times = (C.c_double * 256)()
        stat = (C.c_int32 * 256)()
        gc_was_enabled = gc.isenabled()
        gc.disable()
        try:
            t0 = time.monotonic()
            nxt, done = 0, 0
            while done < len(prepared):
                now = time.monotonic() - t0
                if now > timeout_s:
                    raise TimeoutError(f"serving run exceeded {timeout_s} s")
                while nxt < len(prepared) and prepared[nxt][0].arrival <= now:
                    jid = _lib.check(int(submit(prepared[nxt])))
                    prepared[nxt][0].admitted = now
                    byid[jid] = prepared[nxt]
                    nxt += 1
                n = _lib.check(int(self.lib.sarbp_queue_completed(self._q, ids, times, stat,
                                                                  256)))
                for k in range(n):
                    item = byid.pop(ids[k])
                    _lib.check(int(stat[k]))
                    item[0].finished = times[k] - t0
                    finished(item)
                done += n
                if n == 0 and idle_sleep:
                    wait = idle_sleep
                    if nxt < len(prepared):
                        wait = min(wait, max(0.0, prepared[nxt][0].arrival - now))
                    time.sleep(wait)
            wall = time.monotonic() - t0
        finally:
            if gc_was_enabled:
                gc.enable()
        after = self.stats()
        rep = ServingReport(jobs=jobs, wall_s=wall, waves=after["waves"] - before["waves"],
                            gpu_launches=after["launches"] - before["launches"], peak_bytes=0)
        rep.h2d_bytes = after["h2d_bytes"] - before["h2d_bytes"]
        rep.d2h_bytes = after["d2h_bytes"] - before["d2h_bytes"]
        return rep

    def stats(self) -> dict:
        """The queue's totals (sarbp_queue_stats)."""
        v = (C.c_int64 * 5)()
        _lib.check(self.lib.sarbp_queue_stats(self._q, v))
        return dict(zip(("jobs", "waves", "launches", "h2d_bytes", "d2h_bytes"), list(v)))

    def close(self) -> None:
        if self._q:
            rc = int(self.lib.sarbp_queue_destroy(self._q))
            self._q = C.c_void_p()
            _lib.check(rc)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
