"""The reference's on-disk formats: headerless little-endian column-major .dat.

Inputs (sar_focuser_puntual_noui.py:334-407): DEM x/y/z ``Dem_{x,y,z}_Dbl<D0>x<D1>.dat``
(float64), trajectory ``Traiett_{x,y,z}_Dbl<Naz>.dat`` (float64),
``Index_Long_<D0>x<D1>.dat`` (int32), ``Mask_Byte_<D0>x<D1>.dat`` (uint8),
``Sint_Long_<D0>x<D1>.dat`` (int32), ``RawData_Cmplx_<Nra>x<Naz>.dat``
(complex64 as interleaved float32 pairs, (Nra, Naz) column-major) and the
scalars ``{NearRange,DeltaRange,Lambda}Dbl_1_elemento.dat`` (one float64).

Outputs: ``SlcMatr_real.dat`` / ``SlcMatr_imag.dat`` (float64, column-major;
README.md:103-104, read by img_visualizer.py:19-21 as (D1, D0) C-order, the
same bytes), ``SlcMatr_complex.dat`` (its format is unspecified in the
reference, README.md:105; here interleaved complex128, column-major), and
the files the reference scripts actually write: ``<base>_SplitF32.dat``
(all real float32 then all imaginary), ``<base>_InterleavedF32.dat`` and
``<base>.npy`` (complex128) -- sar_focuser_puntual_noui.py:440-469.

RawData loaders mirror the three behaviours of the reference:
* ``load_raw_strict``: the CPU script's (sar_focuser_puntual_noui.py:377-400):
  interleaved if the float count is 2*Nra*Naz, else IOError (its split-format
  branch repeats the same size test and can never run; split files are
  accepted here only when asked for explicitly with ``fmt="split"``);
* ``load_raw_data``: the small-GPU script's tolerant loader
  (gpu_small_dataset.py:368-451): drops a trailing odd float, re-derives Naz
  from Nra, else the nearest factor pair, else truncates;
* ``validate_raw_dims``: the large-scene driver's memmap check
  (main_gpu.py:208-248): size must be a multiple of 8 bytes; a mismatch is
  reconciled by Nra or by Naz, else ValueError.
"""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np

DEM_NAMES = {"xxg1": "Dem_x_Dbl{d0}x{d1}.dat", "yyg1": "Dem_y_Dbl{d0}x{d1}.dat",
             "zzg1": "Dem_z_Dbl{d0}x{d1}.dat"}
GRID_NAMES = {"Index": ("Index_Long_{d0}x{d1}.dat", np.int32),
              "Mask": ("Mask_Byte_{d0}x{d1}.dat", np.uint8),
              "Sint": ("Sint_Long_{d0}x{d1}.dat", np.int32)}
TRAJ_NAMES = {"wgsx": "Traiett_x_Dbl{naz}.dat", "wgsy": "Traiett_y_Dbl{naz}.dat",
              "wgsz": "Traiett_z_Dbl{naz}.dat"}
RAW_NAME = "RawData_Cmplx_{nra}x{naz}.dat"
SCALAR_NAMES = {"NearRange": "NearRangeDbl_1_elemento.dat",
                "DeltaRange": "DeltaRangeDbl_1_elemento.dat",
                "Lambda": "LambdaDbl_1_elemento.dat"}


def scene_filenames(dim0: int, dim1: int, nra: int, naz: int) -> dict:
    """The 13 input file names of a scene (sar_focuser_puntual_noui.py:334-340)."""
    names = {k: v.format(d0=dim0, d1=dim1) for k, v in DEM_NAMES.items()}
    names.update({k: v[0].format(d0=dim0, d1=dim1) for k, v in GRID_NAMES.items()})
    names.update({k: v.format(naz=naz) for k, v in TRAJ_NAMES.items()})
    names["RawData"] = RAW_NAME.format(nra=nra, naz=naz)
    names.update(SCALAR_NAMES)
    return names


def read_dat(path, dtype, shape=None, order: str = "F") -> np.ndarray:
    """``np.fromfile(path, dtype)`` reshaped in Fortran order when a shape is given."""
    a = np.fromfile(path, dtype=dtype)
    if shape is None:
        return a
    n = int(np.prod(shape))
    if a.size != n:
        raise ValueError(f"{path}: {a.size} {np.dtype(dtype).name} values, expected {n} "
                         f"for shape {tuple(shape)}")
    return a.reshape(shape, order=order)


def write_dat(path, array, dtype=None) -> None:
    """Raw little-endian bytes of ``array`` in Fortran order."""
    a = np.asarray(array)
    if dtype is not None:
        a = a.astype(dtype)
    a.reshape(-1, order="F").astype(a.dtype.newbyteorder("<"), copy=False).tofile(path)


# ---------------------------------------------------------------------------
# RawData


def _complex_from_floats(f32: np.ndarray, nra: int, naz: int, fmt: str) -> np.ndarray:
    if fmt == "interleaved":
        out = np.empty((nra, naz), dtype=np.complex64, order="F")
        out.reshape(-1, order="F").view(np.float32)[:] = f32[: 2 * nra * naz]
        return out
    if fmt == "split":
        n = nra * naz
        out = np.empty((nra, naz), dtype=np.complex64, order="F")
        flat = out.reshape(-1, order="F")
        flat.real = f32[:n]
        flat.imag = f32[n: 2 * n]
        return out
    raise ValueError(f"unknown RawData format {fmt!r}")


def load_raw_strict(path, nra: int, naz: int, fmt: str = "interleaved") -> np.ndarray:
    """CPU-script semantics: exactly 2*Nra*Naz float32 values, else IOError."""
    f32 = np.fromfile(path, dtype=np.float32)
    expected = 2 * nra * naz
    if f32.size != expected:
        raise IOError(f"RawData file size ({f32.size} floats) does not match expected size for "
                      f"interleaved or split format ({expected} floats).")
    return _complex_from_floats(f32, nra, naz, fmt)


def load_raw_data(data_dir, filename, expected_nra: int, expected_naz: int,
                  fmt: str = "interleaved"):
    """Tolerant loader (gpu_small_dataset.py:368-451); returns (RawData, Nra, Naz)."""
    path = os.path.join(data_dir, filename)
    total_floats = os.path.getsize(path) // 4
    f32 = np.fromfile(path, dtype=np.float32, count=total_floats)
    if f32.size % 2:
        f32 = f32[:-1]                                  # :384-390 drop the odd float
    total_complex = f32.size // 2
    nra = expected_nra
    if nra > 0 and total_complex % nra == 0:
        naz = total_complex // nra                      # :403-405
    else:
        factor = int(math.isqrt(total_complex))         # :410-420 nearest factor pair
        while factor > 1 and total_complex % factor:
            factor -= 1
        if factor > 1:
            nra, naz = factor, total_complex // factor
        else:                                           # :422-427 truncate
            nra = expected_nra
            naz = total_complex // nra
            f32 = f32[: 2 * nra * naz]
    return _complex_from_floats(f32, nra, naz, fmt), nra, naz


def validate_raw_dims(path, expected_nra: int, expected_naz: int) -> tuple[int, int]:
    """Memmap validation (main_gpu.py:208-248); returns (Nra, Naz)."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"Raw data file not found: {path}")
    size = os.path.getsize(path)
    if size % 8:
        raise ValueError(f"RawData file size ({size}) is not a multiple of complex64 size (8 "
                         "bytes)")
    total = size // 8
    nra, naz = expected_nra, expected_naz
    if total != nra * naz:
        if nra > 0 and total % nra == 0:
            naz = total // nra
        elif naz > 0 and total % naz == 0:
            nra = total // naz
        else:
            raise ValueError(f"Could not reconcile file size ({total} complex elements) with "
                             f"expected dimensions {expected_nra}x{expected_naz}")
    return nra, naz


def open_raw_memmap(path, nra: int, naz: int) -> np.memmap:
    """Read-only complex64 (Nra, Naz) column-major memory map (main_gpu.py:375-381)."""
    return np.memmap(path, dtype=np.complex64, mode="r", shape=(nra, naz), order="F")


def reconcile_trajectory(raw, wgsx, wgsy, wgsz):
    """Trajectory / RawData azimuth length reconciliation.

    A shorter trajectory truncates the raw data's pulses, a longer one is
    truncated to the raw data (gpu_small_dataset.py:570-585,
    main_gpu.py:387-398).  Returns (raw, wgsx, wgsy, wgsz).
    """
    naz = raw.shape[1]
    tl = min(len(wgsx), len(wgsy), len(wgsz))
    if tl < naz:
        raw = raw[:, :tl]
    elif tl > naz:
        wgsx, wgsy, wgsz = wgsx[:naz], wgsy[:naz], wgsz[:naz]
    return raw, wgsx, wgsy, wgsz


# ---------------------------------------------------------------------------
# whole scenes


def save_scene(data_dir, scene: dict) -> dict:
    """Write a scene's 13 inputs under their reference file names."""
    d = Path(data_dir)
    d.mkdir(parents=True, exist_ok=True)
    dim0, dim1 = np.shape(scene["xxg1"])
    raw = scene["RawData"]
    nra, naz = (int(v) for v in raw.shape)
    names = scene_filenames(dim0, dim1, nra, naz)
    for k in DEM_NAMES:
        write_dat(d / names[k], scene[k], np.float64)
    for k, (_, dt) in GRID_NAMES.items():
        write_dat(d / names[k], scene[k], dt)
    for k in TRAJ_NAMES:
        write_dat(d / names[k], scene[k], np.float64)
    if hasattr(raw, "detach"):
        # a (Nra, Naz) tensor: the file's column-major bytes are its pulse
        # rows, written in blocks of rows (no whole host copy)
        rows = raw.detach().t()
        with open(d / names["RawData"], "wb") as f:
            step = max(1, (256 << 20) // max(1, 8 * nra))
            for a0 in range(0, naz, step):
                blk = rows[a0:a0 + step].to("cpu").contiguous()
                blk.numpy().astype(np.complex64, copy=False).tofile(f)
    else:
        write_dat(d / names["RawData"], raw, np.complex64)
    for k in SCALAR_NAMES:
        write_dat(d / names[k], np.array([scene[k]], dtype=np.float64))
    return names


def load_scene(data_dir, dim0: int, dim1: int, nra: int, naz: int,
               raw_loader: str = "strict") -> dict:
    """Read a scene's 13 inputs as the reference's CPU script does (:355-407).

    ``raw_loader`` "strict" (CPU script), "tolerant" (small-GPU script, with
    trajectory reconciliation) or "memmap" (large-scene driver).
    """
    d = Path(data_dir)
    names = scene_filenames(dim0, dim1, nra, naz)
    sc = {k: read_dat(d / names[k], np.float64, (dim0, dim1)) for k in DEM_NAMES}
    for k, (_, dt) in GRID_NAMES.items():
        sc[k] = read_dat(d / names[k], dt, (dim0, dim1))
    traj = {k: read_dat(d / names[k], np.float64) for k in TRAJ_NAMES}
    if raw_loader == "strict":
        raw = load_raw_strict(d / names["RawData"], nra, naz)
    elif raw_loader == "tolerant":
        raw, _, _ = load_raw_data(d, names["RawData"], nra, naz)
    elif raw_loader == "memmap":
        n_ra, n_az = validate_raw_dims(d / names["RawData"], nra, naz)
        raw = open_raw_memmap(d / names["RawData"], n_ra, n_az)
    else:
        raise ValueError(f"unknown raw_loader {raw_loader!r}")
    if raw_loader != "strict":
        raw, traj["wgsx"], traj["wgsy"], traj["wgsz"] = reconcile_trajectory(
            raw, traj["wgsx"], traj["wgsy"], traj["wgsz"])
    sc.update(traj)
    sc["RawData"] = raw
    for k, n in SCALAR_NAMES.items():
        sc[k] = np.float64(np.fromfile(d / n, dtype=np.float64)[0])
    return sc


# ---------------------------------------------------------------------------
# focused image


def write_slc(out_dir, image: np.ndarray, base: str = "SlcPx_GB300") -> dict:
    """Write a focused complex image in every format the reference names.

    Returns {format: path}.
    """
    d = Path(out_dir)
    d.mkdir(parents=True, exist_ok=True)
    img = np.asarray(image)
    paths = {
        "real": d / "SlcMatr_real.dat", "imag": d / "SlcMatr_imag.dat",
        "complex": d / "SlcMatr_complex.dat", "split_f32": d / f"{base}_SplitF32.dat",
        "interleaved_f32": d / f"{base}_InterleavedF32.dat", "npy": d / f"{base}.npy",
    }
    write_dat(paths["real"], img.real, np.float64)
    write_dat(paths["imag"], img.imag, np.float64)
    write_dat(paths["complex"], img, np.complex128)
    with open(paths["split_f32"], "wb") as f:
        img.real.astype(np.float32).reshape(-1, order="F").tofile(f)
        img.imag.astype(np.float32).reshape(-1, order="F").tofile(f)
    write_dat(paths["interleaved_f32"], img, np.complex64)
    np.save(paths["npy"], img.astype(np.complex128))
    return {k: str(v) for k, v in paths.items()}


def read_slc(path, shape, fmt: str) -> np.ndarray:
    """Read back an image written by ``write_slc`` (fmt: a key of its result)."""
    n = shape[0] * shape[1]
    if fmt == "npy":
        return np.load(path)
    if fmt == "complex":
        return read_dat(path, np.complex128, shape)
    if fmt == "interleaved_f32":
        return read_dat(path, np.complex64, shape)
    if fmt == "split_f32":
        f = np.fromfile(path, dtype=np.float32)
        if f.size != 2 * n:
            raise ValueError(f"{path}: {f.size} float32 values, expected {2 * n}")
        return (f[:n] + 1j * f[n:]).reshape(shape, order="F")
    if fmt in ("real", "imag"):
        return read_dat(path, np.float64, shape)
    raise ValueError(f"unknown image format {fmt!r}")
