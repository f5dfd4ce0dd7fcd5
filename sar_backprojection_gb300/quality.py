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
compares two images stored as interleaved complex128 (.dat) or .npy files.
"""
from __future__ import annotations

import argparse
import json

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


def phase_stats(a, b, rel_threshold: float = 1e-5) -> dict:
    """Wrapped phase-difference statistics (radians) of a against b."""
    a, b = _np(a), _np(b)
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


def compare(a, b) -> dict:
    """rel-L2, coherence and RMS phase error (mrad) of a against reference b."""
    ps = phase_stats(a, b)
    return {"rel_l2": rel_l2(a, b), "coherence": coherence(a, b),
            "rms_phase_mrad": ps.get("rms_mrad", 0.0), "phase": ps}


def load_image(path: str, shape: tuple[int, int]) -> np.ndarray:
    if path.endswith(".npy"):
        return np.load(path).reshape(shape, order="F")
    flat = np.fromfile(path, dtype=np.complex128)
    if flat.size != shape[0] * shape[1]:
        raise ValueError(f"{path}: {flat.size} complex128 values, expected {shape[0] * shape[1]}")
    return flat.reshape(shape, order="F")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("image")
    ap.add_argument("reference")
    ap.add_argument("--shape", type=int, nargs=2, required=True)
    ns = ap.parse_args(argv)
    a = load_image(ns.image, tuple(ns.shape))
    b = load_image(ns.reference, tuple(ns.shape))
    print(json.dumps(compare(a, b), indent=2))


if __name__ == "__main__":
    main()
