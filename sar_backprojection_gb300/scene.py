"""Device-resident focusing scenes.

A scene is the reference's 13 positional focusing arguments
(sar_focuser_puntual_noui.py:149): DEM x/y/z, mask, index, the trajectory,
the complex64 raw data, near range, range spacing, wavelength and Sint.  On
the device every DEM-grid array is flattened in column-major order (as the
reference flattens them, :183-188) and the raw data are stored pulse-major
with an even row pitch (range bins of one pulse contiguous, rows 16-byte
aligned) -- the reference's own column-major RawData byte order, padded when
Nra is odd.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib


def _host_view(a: np.ndarray) -> torch.Tensor:
    """torch view of a host array's memory.  Read-only arrays (memory maps,
    buffers) are only ever read here, so torch's warning about them is
    silenced."""
    if a.flags.writeable:
        return torch.from_numpy(a)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)
        return torch.from_numpy(a)


def _as_tensor(a) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        return a
    return _host_view(np.asarray(a))


def _cast_host(a, np_dtype):
    """Reference dtype coercion (``astype``) on host arrays; tensors via torch."""
    if isinstance(a, torch.Tensor):
        return a.to(getattr(torch, np.dtype(np_dtype).name))
    a = np.asarray(a)
    return a if a.dtype == np_dtype else a.astype(np_dtype)


def _to_device(t: torch.Tensor, device, sm: bool) -> torch.Tensor:
    """Host tensor -> device tensor on the current stream; with ``sm`` a
    contiguous page-locked source is copied by SM loads
    (sarbp_copy_to_device_sm) instead of a copy engine."""
    if sm and t.device.type == "cpu" and t.is_contiguous() and t.is_pinned():
        d = torch.empty(t.shape, dtype=t.dtype, device=device)
        _lib.check(_lib.load().sarbp_copy_to_device_sm(
            d.data_ptr(), t.data_ptr(), t.numel() * t.element_size(),
            torch.cuda.current_stream(d.device).cuda_stream))
        return d
    return t.to(device, non_blocking=True)


def flatten_f(a, np_dtype, device, sm: bool = False) -> torch.Tensor:
    """``a.astype(dtype).flatten(order='F')`` as a contiguous device tensor."""
    a = _cast_host(a, np_dtype)
    t = _as_tensor(a)
    if t.dim() > 1:
        # C-order flatten of the axis-reversed array == F-order flatten
        t = t.permute(*reversed(range(t.dim())))
    t = _to_device(t, device, sm)
    return t.contiguous().view(-1)


def raw_to_device(raw, device, pitch_multiple: int = 2) -> tuple[torch.Tensor, int, int, int]:
    """Complex64 (Nra, Naz) raw data -> pulse-major float pairs on the device.

    Returns (tensor of shape (Naz, pitch, 2) float32, nra, naz, pitch) where
    sample (r, a) is tensor[a, r].
    """
    if isinstance(raw, torch.Tensor):
        t = raw if raw.dtype == torch.complex64 else raw.to(torch.complex64)
    else:
        arr = np.asarray(raw)
        if arr.dtype != np.complex64:
            arr = arr.astype(np.complex64)
        t = _host_view(arr)
    if t.dim() != 2:
        raise ValueError("Raw_Data must be a 2D array")
    nra, naz = int(t.shape[0]), int(t.shape[1])
    pitch = -(-nra // pitch_multiple) * pitch_multiple
    tt = t.t()                                    # (naz, nra)
    if pitch == nra:
        dev = tt.to(device, non_blocking=True)
        if not dev.is_contiguous():
            dev = dev.contiguous()
        out = torch.view_as_real(dev)
    else:
        out = torch.zeros((naz, pitch, 2), dtype=torch.float32, device=device)
        out[:, :nra, :] = torch.view_as_real(tt.to(device, non_blocking=True))
    return out, nra, naz, pitch


@dataclass
class DeviceScene:
    """One focusing scene resident in device memory."""

    dim0: int
    dim1: int
    x: torch.Tensor
    y: torch.Tensor
    z: torch.Tensor
    mask: torch.Tensor
    index: torch.Tensor
    sint: torch.Tensor
    tx: torch.Tensor
    ty: torch.Tensor
    tz: torch.Tensor
    raw: torch.Tensor          # (naz, pitch, 2) float32
    nra: int
    naz: int
    pitch: int
    near_range: float
    delta_range: float
    lambda_: float
    _struct: _lib.Scene | None = field(default=None, repr=False)
    # raw_bins="reached" uploads: range bins [bin_lo, bin_hi] of every pulse
    # are on the device (the rest of each row is never read), the bytes copied
    # host -> device, and the mixed workspace prepared on the way
    bin_lo: int = 0
    bin_hi: int = -1
    h2d_bytes: int = 0
    workspace: torch.Tensor | None = field(default=None, repr=False)
    host_rows: torch.Tensor | None = field(default=None, repr=False)
    # raw_bins="deferred": pinned int32 pair the bound is copied into
    bound_host: torch.Tensor | None = field(default=None, repr=False)

    @property
    def npix(self) -> int:
        return self.dim0 * self.dim1

    @property
    def device(self) -> torch.device:
        return self.raw.device

    def struct(self) -> _lib.Scene:
        """The C ``sarbp_scene`` view of this scene (device pointers)."""
        if self._struct is None:
            s = _lib.Scene()
            s.dim0, s.dim1 = self.dim0, self.dim1
            s.dem_x, s.dem_y, s.dem_z = self.x.data_ptr(), self.y.data_ptr(), self.z.data_ptr()
            s.mask, s.index, s.sint = (self.mask.data_ptr(), self.index.data_ptr(),
                                       self.sint.data_ptr())
            s.traj_x, s.traj_y, s.traj_z = (self.tx.data_ptr(), self.ty.data_ptr(),
                                            self.tz.data_ptr())
            s.raw = self.raw.data_ptr()
            s.nra, s.naz, s.raw_pitch = self.nra, self.naz, self.pitch
            s.near_range, s.delta_range, s.lambda_ = (self.near_range, self.delta_range,
                                                      self.lambda_)
            self._struct = s
        return self._struct

    def nominal_pixel_pulses(self) -> int:
        """Sum over pixels with mask==1 and Sint != -9999 of ceil(Sint/2)*2+1.

        The implementation-independent unit of work (pixel-pulse back-
        projections), computed from the inputs.
        """
        s = self.sint.to(torch.int64)
        ok = (self.mask == 1) & (self.sint != -9999)
        half = torch.where(s >= 0, (s + 1) // 2, -((-s) // 2))
        jj = half * 2 + 1
        return int(torch.where(ok & (jj > 0), jj, torch.zeros_like(jj)).sum().item())

    def nbytes(self) -> int:
        ts = (self.x, self.y, self.z, self.mask, self.index, self.sint, self.tx, self.ty,
              self.tz, self.raw)
        return sum(t.numel() * t.element_size() for t in ts)


def _pulse_major_host(raw):
    """(Naz, Nra) C-contiguous complex64 host view of an F-order (Nra, Naz)
    raw array, or None when the host layout does not allow it."""
    if isinstance(raw, torch.Tensor):
        if raw.device.type != "cpu" or raw.dtype != torch.complex64:
            return None
        t = raw.t()
    else:
        a = np.asarray(raw)
        if a.dtype != np.complex64 or not a.flags.f_contiguous:
            return None
        t = _host_view(a.T)
    return t if t.is_contiguous() else None


def _upload_reached_bins(scene: "DeviceScene", host_rows: torch.Tensor, upload: bool = True,
                         tuning=None) -> None:
    """Copy only the range bins the focusing can read (sarbp_raw_bin_range)
    of every pulse row into the scene's (uninitialised) raw buffer; with
    ``upload=False`` only the bound is computed (the caller copies)."""
    from .focuser import resolve_tuning
    lib = _lib.load()
    dev = scene.device
    stream = torch.cuda.current_stream(dev).cuda_stream
    t = resolve_tuning(tuning)
    sc = C.byref(scene.struct())
    need = _lib.check(int(lib.sarbp_mixed_workspace_size(sc, C.byref(t))))
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    _lib.check(lib.sarbp_mixed_prepare(sc, C.byref(t), ws.data_ptr(), need, stream))
    rng = (C.c_int64 * 2)()
    _lib.check(lib.sarbp_raw_bin_range(sc, C.byref(t), ws.data_ptr(), need, rng, stream))
    lo, hi = int(rng[0]), int(rng[1])
    if upload and hi >= lo:
        _lib.check(lib.sarbp_upload_raw_bins(scene.raw.data_ptr(), scene.pitch,
                                             host_rows.data_ptr(), scene.nra, lo, hi - lo + 1,
                                             scene.naz, stream))
    scene.bin_lo, scene.bin_hi = lo, hi
    if upload:
        scene.h2d_bytes += max(0, hi - lo + 1) * scene.naz * 8
    scene.workspace = ws


def _bound_reached_bins_async(scene: "DeviceScene", bound_host: torch.Tensor,
                              tuning=None) -> None:
    """Enqueue the chunk tables and the reachable-bin bound with its copy
    into ``bound_host`` (pinned int32[2], sarbp_raw_bin_range_async) on the
    current stream, without waiting for it; ``read_bound`` takes it once the
    stream has passed."""
    from .focuser import resolve_tuning
    lib = _lib.load()
    dev = scene.device
    stream = torch.cuda.current_stream(dev).cuda_stream
    t = resolve_tuning(tuning)
    sc = C.byref(scene.struct())
    need = _lib.check(int(lib.sarbp_mixed_workspace_size(sc, C.byref(t))))
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    _lib.check(lib.sarbp_mixed_prepare(sc, C.byref(t), ws.data_ptr(), need, stream))
    _lib.check(lib.sarbp_raw_bin_range_async(sc, C.byref(t), ws.data_ptr(), need,
                                             bound_host.data_ptr(), stream))
    scene.workspace = ws
    scene.bound_host = bound_host


def read_bound(scene: "DeviceScene") -> tuple[int, int]:
    """The bound a raw_bins="deferred" upload enqueued, as (bin_lo, bin_hi)
    (bin_lo > bin_hi: no bin is reached); call it once the stream the scene
    was uploaded on has passed the bound (an event recorded after the upload
    has completed)."""
    if scene.bound_host is not None:
        scene.bin_lo, scene.bin_hi = int(scene.bound_host[0]), int(scene.bound_host[1])
        scene.bound_host = None
    return scene.bin_lo, scene.bin_hi


def scene_to_device(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data,
                    near_range, dra, lambda_val, Sint, device=None,
                    raw_bins: str = "all", tuning=None,
                    raw_buffer: torch.Tensor | None = None,
                    bound_host: torch.Tensor | None = None,
                    h2d: str = "copy") -> DeviceScene:
    """Upload the reference's 13 focusing arguments (same order) to the device.

    Raises ValueError where the reference does (Raw_Data or xxg1 not 2-D,
    sar_focuser_puntual_noui.py:163-170) and for arrays whose sizes do not
    match the DEM grid or a trajectory shorter than Naz (where the reference
    would fail with an IndexError inside its pixel loop).

    ``raw_bins="reached"``: when the raw data are a host array in the
    reference's column-major layout, only the range bins some pixel's
    aperture can reach are copied (a bound computed on the device from the
    DEM, apertures and trajectory, with margins); the kernels never read the
    rest of the device buffer.  Other layouts, and device inputs, are taken
    whole.  ``raw_bins="bound"``: the same bound, but no raw row is copied
    (the caller streams them; ``scene.host_rows`` is the host source) and
    ``scene.workspace`` holds tables prepared with ``tuning``.
    ``raw_bins="deferred"``: as "bound", but the bound is not waited for: it
    is copied into ``bound_host`` (pinned int32[2]) in stream order and
    ``read_bound`` takes it later.
    ``raw_buffer``: a float32 (Naz, pitch, 2) device tensor to receive the
    raw rows in those modes instead of a new allocation (the caller owns
    its reuse).
    ``h2d="sm"``: page-locked host inputs other than the raw rows are copied
    by SM loads instead of a copy engine (``sarbp_copy_to_device_sm``).
    """
    if h2d not in ("copy", "sm"):
        raise ValueError(f"h2d must be 'copy' or 'sm', got {h2d!r}")
    sm = h2d == "sm"
    if raw_bins not in ("all", "reached", "bound", "deferred"):
        raise ValueError("raw_bins must be 'all', 'reached', 'bound' or 'deferred', "
                         f"got {raw_bins!r}")
    if raw_bins == "deferred" and bound_host is None:
        raise ValueError("raw_bins='deferred' needs a pinned int32[2] bound_host")
    raw_shape = tuple(Raw_Data.shape)
    if len(raw_shape) != 2:
        raise ValueError("Raw_Data must be a 2D array")
    if len(tuple(xxg1.shape)) != 2:
        raise ValueError("xxg1 must be a 2D array")
    dim0, dim1 = (int(v) for v in xxg1.shape)
    npix = dim0 * dim1
    nra, naz = (int(v) for v in raw_shape)
    for name, a in (("yyg1", yyg1), ("zzg1", zzg1), ("mask", mask), ("index", index),
                    ("Sint", Sint)):
        size = int(np.prod(tuple(a.shape)))
        if size != npix:
            raise ValueError(f"{name} has {size} elements, the DEM grid has {npix}")
    # the reference reads the trajectory only at pulses 0 < a < Naz-1
    # (sar_focuser_puntual_noui.py:46-55, :71-73): Naz-1 points suffice
    for name, w in (("wgsx", wgsx), ("wgsy", wgsy), ("wgsz", wgsz)):
        if int(np.prod(tuple(w.shape))) < naz - 1:
            raise ValueError(f"{name} has fewer than the {naz - 1} points Raw_Data's {naz} "
                             "pulses need")

    if not torch.cuda.is_available():
        raise RuntimeError("sar_backprojection_gb300 needs a CUDA device (no CPU fallback)")
    device = (torch.device(device) if device is not None
              else torch.device("cuda", torch.cuda.current_device()))
    host_rows = _pulse_major_host(Raw_Data) if raw_bins != "all" else None
    if host_rows is not None:
        pitch = nra + (nra & 1)
        if (raw_buffer is not None and tuple(raw_buffer.shape) == (naz, pitch, 2)
                and raw_buffer.dtype == torch.float32 and raw_buffer.device == device):
            raw_t = raw_buffer
        else:
            raw_t = torch.empty((naz, pitch, 2), dtype=torch.float32, device=device)
    else:
        raw_t, nra, naz, pitch = raw_to_device(Raw_Data, device)

    def traj(w):
        t = _as_tensor(_cast_host(w, np.float64)).reshape(-1)
        if t.numel() < naz:
            # pulse Naz-1 never contributes; the mixed path's per-pulse tables
            # still span every pulse, so repeat the last point for it
            pad = (t[-1:] if t.numel() else torch.zeros(1, dtype=t.dtype)).expand(naz - t.numel())
            t = torch.cat([t, pad])
        return _to_device(t, device, sm).contiguous()

    scene = DeviceScene(
        dim0=dim0, dim1=dim1,
        x=flatten_f(xxg1, np.float64, device, sm), y=flatten_f(yyg1, np.float64, device, sm),
        z=flatten_f(zzg1, np.float64, device, sm),
        mask=flatten_f(mask, np.uint8, device, sm), index=flatten_f(index, np.int32, device, sm),
        sint=flatten_f(Sint, np.int32, device, sm),
        tx=traj(wgsx), ty=traj(wgsy), tz=traj(wgsz),
        raw=raw_t, nra=nra, naz=naz, pitch=pitch,
        near_range=float(near_range), delta_range=float(dra), lambda_=float(lambda_val),
    )
    small = sum(t.numel() * t.element_size() for t in (scene.x, scene.y, scene.z, scene.mask,
                                                        scene.index, scene.sint, scene.tx,
                                                        scene.ty, scene.tz))
    if host_rows is not None:
        scene.h2d_bytes = small
        if raw_bins == "deferred":
            _bound_reached_bins_async(scene, bound_host, tuning=tuning)
        else:
            _upload_reached_bins(scene, host_rows, upload=raw_bins == "reached", tuning=tuning)
        scene.host_rows = host_rows if raw_bins in ("bound", "deferred") else None
    else:
        scene.bin_lo, scene.bin_hi = 0, nra - 1
        scene.h2d_bytes = small + (nra * naz * 8 if Raw_Data is not None and
                                   not (isinstance(Raw_Data, torch.Tensor) and
                                        Raw_Data.device.type == "cuda") else 0)
    return scene
