"""Seeded synthetic focusing scenes for the benchmark workloads.

The reference ships no data (its .dat inputs are git-ignored), so every
workload is a seeded synthetic scene with the reference's array shapes,
dtypes and column-major layout:

* ``config_small``: 256 x 64 flat DEM at 1 m, 2001 pulses at 0.5 m with
  N(0, 0.02 m) along-track jitter, Nra = 512, 8 point targets + 20 dB noise,
  Sint = 400, all-ones mask (CPU-runnable; the oracle's full case).
* ``config_full``: 4000 x 250 DEM (5 m azimuth x 4 m range) over seeded
  Gaussian terrain (sigma 30 m, 200 m correlation), 40001 pulses at 0.5 m with
  low-frequency motion within +-1 m, Nra = 4762 (1.52 GB of raw data),
  200 point targets + slope-weighted circular Gaussian clutter, Sint linear in
  range index from 1200 to 1800, 80 % mask in seeded blobs.
* ``uneven_specs``: 48 scenes with log-uniform sizes (DEM 128 x 32 ..
  2000 x 250, 2001 .. 20001 pulses, Sint 200 .. 1800), each built like
  ``config_full`` at its own size.

Geometry: azimuth along x, sensor track at y = -2000 m, z = 3000 m, ground
range along +y.  The echo model is a range sinc times exp(-j*4*pi*R/lambda)
(no chirp term, so targets defocus slightly under the reference's beta*R^2
phase; parity compares implementations, not image quality).

Geometry and small-scene raw data are generated with NumPy; the raw data of
large scenes are synthesised with torch (on the GPU when one is present).
"""
from __future__ import annotations

import hashlib
import math
from dataclasses import dataclass, replace

import numpy as np

C_LIGHT = 2.9979246e8


@dataclass(frozen=True)
class SceneSpec:
    """Parameters of one synthetic scene (all lengths in metres)."""

    name: str = "scene"
    seed: int = 0
    dim0: int = 256            # azimuth pixels (first DEM axis)
    dim1: int = 64             # range pixels (second DEM axis)
    az_spacing: float = 1.0
    rg_spacing: float = 1.0
    x0: float = 372.0          # x of pixel row 0
    y0: float = 50.0           # ground y of range column 0
    terrain_sigma: float = 0.0
    terrain_corr: float = 200.0
    naz: int = 2001
    pulse_spacing: float = 0.5
    jitter_sigma: float = 0.02     # white along-track jitter (config_small)
    motion_amp: float = 0.0        # low-frequency motion bound (config_full)
    track_y: float = -2000.0
    track_z: float = 3000.0
    nra: int = 512
    near_range: float = 3550.0
    delta_range: float = 0.5
    wavelength: float = 0.031
    n_targets: int = 8
    snr_db: float | None = 20.0    # white noise relative to signal power
    clutter: bool = False          # slope-weighted clutter (config_full)
    sint_lo: int = 400
    sint_hi: int = 400             # Sint linear in range index lo -> hi
    mask_fraction: float = 1.0     # fraction of ones, in blobs when < 1
    echo_halfwidth: int = 0        # 0: full-length sinc; else +- bins


def config_small(seed: int = 1) -> SceneSpec:
    return SceneSpec(name="small_256x64_2001", seed=seed)


def config_full(seed: int = 2) -> SceneSpec:
    return SceneSpec(
        name="full_4000x250_40001", seed=seed, dim0=4000, dim1=250, az_spacing=5.0,
        rg_spacing=4.0, x0=2.5, y0=100.0, terrain_sigma=30.0, terrain_corr=200.0,
        naz=40001, pulse_spacing=0.5, jitter_sigma=0.0, motion_amp=1.0, nra=4762,
        near_range=3500.0, delta_range=0.5, wavelength=0.031, n_targets=200,
        snr_db=None, clutter=True, sint_lo=1200, sint_hi=1800, mask_fraction=0.8,
        echo_halfwidth=8)


def scaled_full(seed: int, dim0: int, dim1: int, naz: int, sint_lo: int, sint_hi: int,
                name: str | None = None) -> SceneSpec:
    """A ``config_full``-like scene at its own size (uneven batch / serving).

    The DEM spans the whole track in azimuth (dim0 pixels over naz pulses) and
    keeps the 4 m ground-range spacing (a dim1 x 4 m swath)."""
    track = 0.5 * (naz - 1)
    az = track / dim0
    return replace(config_full(seed), name=name or f"scene_{dim0}x{dim1}_{naz}", dim0=dim0,
                   dim1=dim1, az_spacing=az, x0=0.5 * az, naz=naz, sint_lo=sint_lo,
                   sint_hi=sint_hi, rg_spacing=4.0,
                   n_targets=max(8, int(200 * dim0 * dim1 / 1.0e6)))


def large_spec(seed: int = 6, dim_az: int = 32000, dim_rg: int = 4000, naz: int = 403484,
               n_targets: int = 2000) -> SceneSpec:
    """The reference's large-scene size (DEM 4000 x 32000, RawData 4762 x
    403484 = 15.4 GB; main_gpu.py:321-324) with config_full's physics.

    Azimuth is the first axis of the generated grid (``azimuth_columns``
    turns it into the reference's (DimRg, DimAz) layout): dim_az pixels over
    the whole track, dim_rg range pixels at 0.7 m ground spacing (slant
    ranges 3.6-5.8 km inside the 4762-bin swath)."""
    track = 0.5 * (naz - 1)
    az = track / dim_az
    return replace(config_full(seed), name=f"large_{dim_rg}x{dim_az}_{naz}", dim0=dim_az,
                   dim1=dim_rg, az_spacing=az, x0=0.5 * az, rg_spacing=0.7, naz=naz,
                   n_targets=n_targets)


def uneven_specs(n: int = 48, seed: int = 4) -> list[SceneSpec]:
    """Scenes with log-uniform sizes: DEM 128x32..2000x250, 2001..20001 pulses,
    Sint 200..1800."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        u = rng.random(4)
        dim0 = int(round(math.exp(math.log(128) + u[0] * math.log(2000 / 128))))
        dim1 = int(round(math.exp(math.log(32) + u[1] * math.log(250 / 32))))
        naz = int(round(math.exp(math.log(2001) + u[2] * math.log(20001 / 2001))))
        naz |= 1
        s_hi = int(round(math.exp(math.log(200) + u[3] * math.log(1800 / 200))))
        s_lo = max(200, int(s_hi * 0.67))
        out.append(scaled_full(seed * 1000 + i, dim0, dim1, naz, s_lo, s_hi,
                               name=f"uneven{i:02d}_{dim0}x{dim1}_{naz}"))
    return out


# --------------------------------------------------------------------------
# geometry


def _smooth_field(rng, shape, spacing0, spacing1, corr):
    """Unit-variance Gaussian random field with Gaussian correlation length."""
    w = rng.standard_normal(shape)
    k0 = np.fft.fftfreq(shape[0], d=spacing0)
    k1 = np.fft.rfftfreq(shape[1], d=spacing1)
    kk = k0[:, None] ** 2 + k1[None, :] ** 2
    filt = np.exp(-0.5 * (2 * np.pi) ** 2 * kk * (corr / 2) ** 2)
    f = np.fft.irfft2(np.fft.rfft2(w) * filt, s=shape)
    f -= f.mean()
    sd = f.std()
    return f / sd if sd > 0 else f


def trajectory(spec: SceneSpec, rng) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    k = np.arange(spec.naz, dtype=np.float64)
    x = spec.pulse_spacing * k
    y = np.full(spec.naz, spec.track_y)
    z = np.full(spec.naz, spec.track_z)
    if spec.jitter_sigma > 0:
        x = x + rng.normal(0.0, spec.jitter_sigma, spec.naz)
    if spec.motion_amp > 0:
        L = max(spec.pulse_spacing * (spec.naz - 1), 1.0)
        for comp in (0, 1, 2):
            m = np.zeros(spec.naz)
            for _ in range(4):
                wl = rng.uniform(0.2, 1.0) * L
                m += rng.uniform(0.3, 1.0) * np.sin(2 * np.pi * k * spec.pulse_spacing / wl
                                                    + rng.uniform(0, 2 * np.pi))
            m *= spec.motion_amp / max(np.abs(m).max(), 1e-12)
            if comp == 0:
                x = x + 0.5 * m
            elif comp == 1:
                y = y + m
            else:
                z = z + m
    return x, y, z


def nearest_pulse(traj_x: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Index of the pulse nearest each x (trajectory x increasing)."""
    i = np.clip(np.searchsorted(traj_x, x), 1, len(traj_x) - 1)
    left = traj_x[i - 1]
    right = traj_x[i]
    return np.where(np.abs(x - left) <= np.abs(right - x), i - 1, i).astype(np.int32)


def geometry(spec: SceneSpec) -> dict:
    """DEM, trajectory, Index, Sint and Mask (column-major arrays)."""
    rng = np.random.default_rng(spec.seed)
    i = np.arange(spec.dim0, dtype=np.float64)
    j = np.arange(spec.dim1, dtype=np.float64)
    xg = spec.x0 + spec.az_spacing * i
    yg = spec.y0 + spec.rg_spacing * j
    xx = np.asfortranarray(np.repeat(xg[:, None], spec.dim1, axis=1))
    yy = np.asfortranarray(np.repeat(yg[None, :], spec.dim0, axis=0))
    if spec.terrain_sigma > 0:
        zz = spec.terrain_sigma * _smooth_field(rng, (spec.dim0, spec.dim1), spec.az_spacing,
                                                spec.rg_spacing, spec.terrain_corr)
    else:
        zz = np.zeros((spec.dim0, spec.dim1))
    zz = np.asfortranarray(zz)
    tx, ty, tz = trajectory(spec, rng)
    index = np.asfortranarray(np.repeat(nearest_pulse(tx, xg)[:, None], spec.dim1, axis=1))
    if spec.dim1 > 1:
        srow = spec.sint_lo + (spec.sint_hi - spec.sint_lo) * j / (spec.dim1 - 1)
    else:
        srow = np.full(1, float(spec.sint_lo))
    sint = np.asfortranarray(np.repeat(np.rint(srow).astype(np.int32)[None, :], spec.dim0,
                                       axis=0))
    if spec.mask_fraction >= 1.0:
        mask = np.ones((spec.dim0, spec.dim1), dtype=np.uint8)
    else:
        f = _smooth_field(rng, (spec.dim0, spec.dim1), spec.az_spacing, spec.rg_spacing, 150.0)
        thr = np.quantile(f, 1.0 - spec.mask_fraction)
        mask = (f > thr).astype(np.uint8)
    mask = np.asfortranarray(mask)
    return dict(xxg1=xx, yyg1=yy, zzg1=zz, Mask=mask, Index=index, Sint=sint,
                wgsx=tx, wgsy=ty, wgsz=tz, rng=rng)


def _targets(spec: SceneSpec, g: dict, rng) -> tuple[np.ndarray, np.ndarray]:
    ii = rng.integers(0, spec.dim0, spec.n_targets)
    jj = rng.integers(0, spec.dim1, spec.n_targets)
    pos = np.stack([g["xxg1"][ii, jj], g["yyg1"][ii, jj], g["zzg1"][ii, jj]], axis=1)
    amp = rng.uniform(0.5, 1.5, spec.n_targets)
    return pos, amp


# --------------------------------------------------------------------------
# raw data


def _raw_numpy(spec: SceneSpec, g: dict, rng) -> np.ndarray:
    """Full-sinc echoes + white noise, all in NumPy (small scenes)."""
    pos, amp = _targets(spec, g, rng)
    traj = np.stack([g["wgsx"], g["wgsy"], g["wgsz"]], axis=1)
    rbin = spec.near_range + spec.delta_range * np.arange(spec.nra)
    sig = np.zeros((spec.nra, spec.naz), dtype=np.complex128)
    for p, a in zip(pos, amp):
        R = np.sqrt(((traj - p) ** 2).sum(axis=1))
        env = np.sinc((rbin[:, None] - R[None, :]) / spec.delta_range)
        sig += a * env * np.exp(-1j * (4 * np.pi / spec.wavelength) * R)[None, :]
    if spec.snr_db is not None:
        ps = np.mean(np.abs(sig) ** 2)
        sd = math.sqrt(ps / 10 ** (spec.snr_db / 10) / 2)
        sig += sd * (rng.standard_normal(sig.shape) + 1j * rng.standard_normal(sig.shape))
    return np.asfortranarray(sig.astype(np.complex64))


def _raw_torch(spec: SceneSpec, g: dict, rng, device):
    """Truncated-sinc echoes + slope-weighted clutter synthesised with torch.

    Returns a complex64 tensor of shape (nra, naz) whose storage is pulse-
    major (the column-major layout of the reference's RawData file).
    """
    import torch

    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(spec.seed) * 7919 + 17)
    pos, amp = _targets(spec, g, rng)
    tx = torch.as_tensor(g["wgsx"], device=dev)
    ty = torch.as_tensor(g["wgsy"], device=dev)
    tz = torch.as_tensor(g["wgsz"], device=dev)
    naz, nra = spec.naz, spec.nra
    raw = torch.zeros((naz, nra), dtype=torch.complex64, device=dev)   # pulse-major
    if spec.clutter:
        # clutter std per (pulse, bin): 0.5 + 5*|grad z| at the flat-earth
        # ground point of the bin, on the DEM row nearest the pulse.
        zz = g["zzg1"]
        gz0, gz1 = np.gradient(zz, spec.az_spacing, spec.rg_spacing)
        amp_map = torch.as_tensor(0.5 + 5.0 * np.hypot(gz0, gz1), device=dev,
                                  dtype=torch.float32)
        rr = spec.near_range + spec.delta_range * torch.arange(nra, device=dev,
                                                               dtype=torch.float64)
        h = spec.track_z
        ground = torch.sqrt(torch.clamp(rr * rr - h * h, min=0.0)) + spec.track_y
        col = torch.round((ground - spec.y0) / spec.rg_spacing).long()
        col_ok = (col >= 0) & (col < spec.dim1)
        col = col.clamp(0, spec.dim1 - 1)
        row = torch.round((tx - spec.x0) / spec.az_spacing).long()
        row_ok = (row >= 0) & (row < spec.dim0)
        row = row.clamp(0, spec.dim0 - 1)
        blk = 2048
        for a0 in range(0, naz, blk):
            a1 = min(naz, a0 + blk)
            sd = amp_map[row[a0:a1]][:, col]
            ok = row_ok[a0:a1, None] & col_ok[None, :]
            sd = torch.where(ok, sd, torch.full_like(sd, 0.5)) * (0.5 ** 0.5)
            n = torch.randn((a1 - a0, nra, 2), generator=gen, device=dev, dtype=torch.float32)
            raw[a0:a1] = torch.view_as_complex(n * sd[..., None])
    # point targets: +-echo_halfwidth bins of sinc around the target range,
    # pulses within +-1000 of the target's nearest pulse.
    hw = spec.echo_halfwidth or nra
    tscale = 10.0 if spec.clutter else 1.0
    for p, a in zip(pos, amp):
        k_c = int(nearest_pulse(g["wgsx"], np.array([p[0]]))[0])
        k_lo, k_hi = max(0, k_c - 1000), min(naz, k_c + 1001)
        R = torch.sqrt((tx[k_lo:k_hi] - p[0]) ** 2 + (ty[k_lo:k_hi] - p[1]) ** 2
                       + (tz[k_lo:k_hi] - p[2]) ** 2)
        fb = (R - spec.near_range) / spec.delta_range
        b0 = torch.round(fb).long()
        offs = torch.arange(-hw, hw + 1, device=dev)
        bins = b0[:, None] + offs[None, :]
        ok = (bins >= 0) & (bins < nra)
        env = torch.sinc(bins.double() - fb[:, None])
        ph = -(4 * math.pi / spec.wavelength) * R
        val = (tscale * a) * env * torch.exp(1j * ph)[:, None]
        kk = torch.arange(k_lo, k_hi, device=dev)[:, None].expand_as(bins)
        raw.index_put_((kk[ok], bins[ok]), val[ok].to(torch.complex64), accumulate=True)
    if spec.snr_db is not None and not spec.clutter:
        ps = float((raw.abs() ** 2).mean())
        sd = math.sqrt(ps / 10 ** (spec.snr_db / 10) / 2)
        n = torch.randn((naz, nra, 2), generator=gen, device=dev, dtype=torch.float32) * sd
        raw += torch.view_as_complex(n)
    return raw.t()     # (nra, naz) view, pulse-major storage


def generate(spec: SceneSpec, raw_device: str | None = None) -> dict:
    """Generate the reference's 13 focusing inputs for ``spec``.

    Returns a dict with keys xxg1, yyg1, zzg1, Mask, Index, wgsx, wgsy, wgsz,
    RawData, NearRange, DeltaRange, Lambda, Sint.  ``raw_device`` None uses
    NumPy for the raw data (complex64 (Nra, Naz), column-major); otherwise the
    raw data are a torch complex64 (Nra, Naz) tensor on that device.
    """
    g = geometry(spec)
    rng = g.pop("rng")
    if raw_device is None:
        raw = _raw_numpy(spec, g, rng)
    else:
        raw = _raw_torch(spec, g, rng, raw_device)
    g.update(RawData=raw, NearRange=np.float64(spec.near_range),
             DeltaRange=np.float64(spec.delta_range), Lambda=np.float64(spec.wavelength))
    return g


def focus_args(scene: dict) -> tuple:
    """The reference's positional argument tuple (sar_focuser_puntual_noui.py:436)."""
    return (scene["xxg1"], scene["yyg1"], scene["zzg1"], scene["Mask"], scene["Index"],
            scene["wgsx"], scene["wgsy"], scene["wgsz"], scene["RawData"],
            scene["NearRange"], scene["DeltaRange"], scene["Lambda"], scene["Sint"])


def nominal_pixel_pulses(scene: dict) -> int:
    """Sum over pixels with Mask == 1 and Sint != -9999 of ceil(Sint/2)*2+1."""
    s = np.asarray(scene["Sint"], dtype=np.int64)
    ok = (np.asarray(scene["Mask"]).astype(np.uint8) == 1) & (s != -9999)
    jj = np.where(s >= 0, (s + 1) // 2, -((-s) // 2)) * 2 + 1
    return int(np.where(ok & (jj > 0), jj, 0).sum())


def input_digest(scene: dict) -> str:
    """SHA-256 over the 13 inputs' bytes (column-major), for fixture pinning."""
    h = hashlib.sha256()
    for k in ("xxg1", "yyg1", "zzg1", "Mask", "Index", "wgsx", "wgsy", "wgsz", "RawData",
              "NearRange", "DeltaRange", "Lambda", "Sint"):
        v = scene[k]
        if hasattr(v, "detach"):
            v = v.detach().cpu().numpy()
        a = np.asarray(v)
        h.update(k.encode())
        h.update(np.ascontiguousarray(a.reshape(-1, order="F")).tobytes())
    return h.hexdigest()


def azimuth_columns(scene: dict) -> dict:
    """The same scene with azimuth along the DEM's second axis.

    The large-scene files of the reference are (DimRg, DimAz) grids batched
    by azimuth columns (main_gpu.py:321-324, :415-434); the generators here
    put azimuth first.  Transposes the six DEM-grid arrays (column-major kept);
    trajectory and raw data are unchanged.
    """
    out = dict(scene)
    for k in ("xxg1", "yyg1", "zzg1", "Mask", "Index", "Sint"):
        out[k] = np.asfortranarray(np.asarray(scene[k]).T)
    return out
