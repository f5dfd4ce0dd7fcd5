"""Image-quality metrics of a focused image against a reference image.

* relative L2 error ``||a - b|| / ||b||``;
* complex coherence ``|sum a*conj(b)| / sqrt(sum|a|^2 * sum|b|^2)``;
* wrapped phase difference ``angle(a*conj(b))`` statistics over pixels where
  both amplitudes exceed a threshold: bias, median, standard deviation, RMS,
  range, IQR, percentiles and counts above pi/4, pi/8, pi/16, pi/32 -- the
  statistics of the reference's phase comparison tool (compare_phase.py:40-199,
  amplitude mask :54-58, RMS :91), with its absolute 1e-6 amplitude floor
  replaced by the relative 1e-5*max threshold of choerence_measure.py:196-197
  so that the mask does not depend on the image's scale.

``python -m sar_backprojection_gb300.quality a.dat b.dat --shape D0 D1``
(or the reference tool's spelling, ``--file1 a.dat --file2 b.dat --shape
D0,D1 --fmt1 split --fmt2 truth``) compares two images and prints the
statistics as JSON; ``--out PREFIX`` also writes ``PREFIX_statistics.json``
as compare_phase.py:220-227 does.  Formats (``--fmt1``/``--fmt2``; default
``auto``: .npy by extension, else by file size, complex128 or complex64):

* ``complex128``: interleaved float64 pairs, column-major (``SlcMatr_complex.dat``);
* ``interleaved`` / ``interleaved_f32``: interleaved float32 pairs,
  column-major (``SlcPx_*_InterleavedF32.dat``, sar_focuser_puntual_noui.py:455-466;
  compare_phase.py:8-21);
* ``split`` / ``split_f32``: all real parts then all imaginary parts, float32,
  column-major (``SlcPx_*_SplitF32.dat``, sar_focuser_puntual_noui.py:441-452;
  compare_phase.py:22-29);
* ``truth``: complex64, column-major (compare_phase.py:33-37; the same bytes
  as ``interleaved``);
* ``slcmatr``: the ``SlcMatr_real.dat`` / ``SlcMatr_imag.dat`` float64 pair
  (README's outputs): give either file or their directory;
* ``npy``: a NumPy complex array (``SlcPx_*.npy``).
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np


def _np(a) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    if a.dtype.kind != "c":
        if a.shape and a.shape[-1] == 2 and a.dtype.kind == "f":
            a = np.ascontiguousarray(a, dtype=np.float64).view(np.complex128)[..., 0]
        else:
            a = a.astype(np.complex128)
    return a.astype(np.complex128, copy=False).reshape(-1)


def rel_l2(a, b) -> float:
    a, b = _np(a), _np(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def coherence(a, b) -> float:
    a, b = _np(a), _np(b)
    den = np.sqrt(np.sum(np.abs(a) ** 2) * np.sum(np.abs(b) ** 2))
    return float(np.abs(np.sum(a * np.conj(b))) / den) if den > 0 else 1.0


def phase_stats(a, b, rel_threshold: float | None = 1e-5) -> dict:
    """Wrapped phase-difference statistics (radians) of a against b.

    ``rel_threshold`` None keeps every pixel (the reference tool's
    ``--no-mask``)."""
    a, b = _np(a), _np(b)
    if rel_threshold is None:
        m = np.ones(a.shape, dtype=bool)
    else:
        amax = max(np.abs(b).max(initial=0.0), np.abs(a).max(initial=0.0))
        thr = rel_threshold * amax
        m = (np.abs(a) > thr) & (np.abs(b) > thr)
    d = np.angle(a[m] * np.conj(b[m]))
    if d.size == 0:
        return {"valid_pixels": 0}
    q = np.percentile(d, [1, 5, 25, 50, 75, 95, 99])
    return {
        "valid_pixels": int(d.size),
        "invalid_pixels": int(m.size - d.size),
        "mean_rad": float(d.mean()),
        "median_rad": float(q[3]),
        "std_rad": float(d.std()),
        "rms_rad": float(np.sqrt(np.mean(d * d))),
        "rms_mrad": float(1e3 * np.sqrt(np.mean(d * d))),
        "min_rad": float(d.min()),
        "max_rad": float(d.max()),
        "iqr_rad": float(q[4] - q[2]),
        "percentiles": {"p1": float(q[0]), "p5": float(q[1]), "p25": float(q[2]),
                        "p75": float(q[4]), "p95": float(q[5]), "p99": float(q[6])},
        "large_errors": {f"pi_{k}": int(np.sum(np.abs(d) > np.pi / k)) for k in (4, 8, 16, 32)},
    }


def compare(a, b, rel_threshold: float | None = 1e-5) -> dict:
    """rel-L2, coherence and RMS phase error (mrad) of a against reference b."""
    ps = phase_stats(a, b, rel_threshold)
    return {"rel_l2": rel_l2(a, b), "coherence": coherence(a, b),
            "rms_phase_mrad": ps.get("rms_mrad", 0.0), "phase": ps}


FORMATS = ("auto", "complex128", "interleaved", "interleaved_f32", "split", "split_f32", "truth",
           "slcmatr", "npy")


def _slcmatr_paths(path: str) -> tuple[str, str]:
    if os.path.isdir(path):
        return (os.path.join(path, "SlcMatr_real.dat"), os.path.join(path, "SlcMatr_imag.dat"))
    d, name = os.path.split(path)
    if "SlcMatr_real" in name:
        return path, os.path.join(d, name.replace("SlcMatr_real", "SlcMatr_imag"))
    if "SlcMatr_imag" in name:
        return os.path.join(d, name.replace("SlcMatr_imag", "SlcMatr_real")), path
    raise ValueError(f"{path}: slcmatr wants SlcMatr_real.dat, SlcMatr_imag.dat or their "
                     "directory")


def load_image(path: str, shape: tuple[int, int], fmt: str = "auto") -> np.ndarray:
    """A complex image of ``shape`` (column-major on disk) in format ``fmt``."""
    from .datfiles import read_dat, read_slc

    if fmt not in FORMATS:
        raise ValueError(f"unknown image format {fmt!r}; one of {FORMATS}")
    n = shape[0] * shape[1]
    if fmt == "auto":
        if path.endswith(".npy"):
            fmt = "npy"
        else:
            size = os.path.getsize(path)
            if size == 16 * n:
                fmt = "complex128"
            elif size == 8 * n:
                fmt = "interleaved"
            else:
                raise ValueError(f"{path}: {size} bytes is neither complex128 nor complex64 for "
                                 f"shape {tuple(shape)}; name the format")
    if fmt == "npy":
        a = np.load(path)
        if a.size != n:
            raise ValueError(f"{path}: {a.size} values, expected {n}")
        return a.reshape(shape, order="F") if a.shape != tuple(shape) else a
    if fmt == "slcmatr":
        re, im = _slcmatr_paths(path)
        return read_dat(re, np.float64, shape) + 1j * read_dat(im, np.float64, shape)
    key = {"complex128": "complex", "interleaved": "interleaved_f32", "truth": "interleaved_f32",
           "split": "split_f32"}.get(fmt, fmt)
    return read_slc(path, shape, key)


def _shape(tokens) -> tuple[int, int]:
    vals = [int(v) for t in tokens for v in str(t).replace(",", " ").split()]
    if len(vals) != 2:
        raise ValueError(f"--shape wants two sizes, got {tokens}")
    return vals[0], vals[1]


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("image", nargs="?")
    ap.add_argument("reference", nargs="?")
    ap.add_argument("--file1", help="image (the reference tool's spelling)")
    ap.add_argument("--file2", help="reference image (the reference tool's spelling)")
    ap.add_argument("--shape", nargs="+", required=True, help="D0 D1 or D0,D1")
    ap.add_argument("--fmt1", default="auto", choices=FORMATS)
    ap.add_argument("--fmt2", default="auto", choices=FORMATS)
    ap.add_argument("--no-mask", action="store_true",
                    help="phase statistics over every pixel (no amplitude threshold)")
    ap.add_argument("--out", default=None, help="also write OUT_statistics.json")
    ns = ap.parse_args(argv)
    f1 = ns.file1 or ns.image
    f2 = ns.file2 or ns.reference
    if not f1 or not f2:
        ap.error("two images are needed (positional or --file1/--file2)")
    shape = _shape(ns.shape)
    a = load_image(f1, shape, ns.fmt1)
    b = load_image(f2, shape, ns.fmt2)
    stats = compare(a, b, None if ns.no_mask else 1e-5)
    text = json.dumps(stats, indent=2)
    print(text)
    if ns.out:
        with open(f"{ns.out}_statistics.json", "w") as f:
            f.write(text + "\n")
    return stats


if __name__ == "__main__":
    main()
