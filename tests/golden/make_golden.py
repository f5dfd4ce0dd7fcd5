"""Generate the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED reference focusing call ``FocalizzatoreBpPx`` from
``sar_focuser_puntual_noui.py`` (read from the reference checkout named by
``--reference DIR`` or, failing that, $SARBP_REFERENCE_DIR) under plain NumPy: numba is not
installed, so a stub module whose ``jit`` returns the function unchanged and
whose ``prange`` is ``range`` is placed in ``sys.modules`` first.  NumPy and
Numba's nopython mode agree on the operations used (IEEE arithmetic, sqrt,
round-half-even, cos/sin via the C library) except that NumPy's
``complex128 / int`` multiplies by the rounded reciprocal; the oracle follows
NumPy, so the fixtures below are bit-exact targets.

Fixtures written (all .npz):
  golden_small.npz  -- the 256 x 64, 2001-pulse small workload: seed, SHA-256
                       of the regenerated inputs and the reference image.
  golden_edges.npz  -- a 24 x 8 scene with every edge case the reference
                       handles (mask 0/1/2/255, Sint -9999/-3/-2/-1/0/odd/even/
                       oversized, Index at 0, 1, Naz-2, Naz-1, outside, range
                       bins across 0 and Nra-2..Nra): inputs and image stored.
  golden_ties.npz   -- exact .5 range-bin ties (half-to-even rounding):
                       inputs and image stored.
  reference_timing.json -- wall time of the reference call on the small
                       workload (one core, NumPy under the numba stub), with
                       the host it ran on: the reference's own CPU speed,
                       which cannot be measured where the reference is absent.

Usage: python tests/golden/make_golden.py --reference DIR [--only small|edges|ties|timing]
"""
from __future__ import annotations

import contextlib
import importlib.util
import io
import json
import os
import platform
import sys
import tempfile
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from sar_backprojection_gb300 import synth  # noqa: E402


def load_reference(ref_dir: str | None):
    """Import the reference module with a numba stub (no files written)."""
    ref_dir = ref_dir or os.environ.get("SARBP_REFERENCE_DIR")
    if not ref_dir:
        raise SystemExit("name the reference checkout: --reference DIR or $SARBP_REFERENCE_DIR")
    ref_dir = Path(ref_dir)
    src = ref_dir / "sar_focuser_puntual_noui.py"
    if not src.exists():
        raise FileNotFoundError(f"reference source not found: {src}")
    stub = types.ModuleType("numba")
    stub.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    stub.prange = range
    sys.modules["numba"] = stub
    sys.dont_write_bytecode = True
    spec = importlib.util.spec_from_file_location("sarbp_reference_cpu", src)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference(mod, scene: dict) -> np.ndarray:
    """Call the reference FocalizzatoreBpPx in a scratch cwd, output silenced."""
    args = synth.focus_args(scene)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                out = mod.FocalizzatoreBpPx(*args)
        finally:
            os.chdir(cwd)
    return np.asarray(out)


def edges_scene(seed: int = 11) -> dict:
    """24 x 8 pixels covering the reference's edge cases."""
    rng = np.random.default_rng(seed)
    dim0, dim1, naz, nra = 24, 8, 301, 80
    near, dra, lam = 3613.7, 0.5, 0.031
    k = np.arange(naz, dtype=np.float64)
    tx = 0.5 * k + rng.normal(0.0, 0.02, naz)
    ty = np.full(naz, -2000.0) + rng.normal(0.0, 0.01, naz)
    tz = np.full(naz, 3000.0)
    xg = 10.0 + 5.0 * np.arange(dim0)                    # 10 .. 125 m along track
    yg = 30.0 + 9.0 * np.arange(dim1)                    # slant ranges across Nra-1
    xx = np.asfortranarray(np.repeat(xg[:, None], dim1, axis=1))
    yy = np.asfortranarray(np.repeat(yg[None, :], dim0, axis=0))
    zz = np.asfortranarray(rng.normal(0.0, 2.0, (dim0, dim1)))
    index = np.asfortranarray(np.repeat(synth.nearest_pulse(tx, xg)[:, None], dim1, axis=1))
    sint = np.asfortranarray(rng.choice([40, 41, 60, 81, 100], size=(dim0, dim1)).astype(np.int32))
    mask = np.ones((dim0, dim1), dtype=np.uint8)
    # explicit edge cases on column 0..3
    sint[0, 0] = -9999
    sint[1, 0] = -3
    sint[2, 0] = -2
    sint[3, 0] = -1
    sint[4, 0] = 0
    sint[5, 0] = 1
    sint[6, 0] = 2
    sint[7, 0] = 3
    sint[8, 0] = 5000                                     # longer than the data
    mask[9, 0] = 0
    mask[10, 0] = 2
    mask[11, 0] = 255
    index[12, 1] = 0
    index[13, 1] = 1
    index[14, 1] = naz - 2
    index[15, 1] = naz - 1
    index[16, 1] = naz + 7
    index[17, 1] = -5
    sint[12:18, 1] = 9
    mask[18, 2] = 0
    sint[18, 2] = -9999
    zz[19:22, 0] = [10.662, 10.672, 10.683]               # range bins across 0
    raw = (rng.standard_normal((nra, naz)) + 1j * rng.standard_normal((nra, naz)))
    raw = np.asfortranarray(raw.astype(np.complex64))
    return dict(xxg1=xx, yyg1=yy, zzg1=zz, Mask=np.asfortranarray(mask), Index=index,
                Sint=sint, wgsx=tx, wgsy=ty, wgsz=tz, RawData=raw,
                NearRange=np.float64(near), DeltaRange=np.float64(dra),
                Lambda=np.float64(lam))


def ties_scene() -> dict:
    """Pixels and pulses whose (R - near)/dra is exactly n + 0.5 in FP64.

    Pulse k sits at (0, 0, z_k) and pixel at (0, 0, 0): R = |z_k| exactly,
    with z_k = near + (n_k + 0.5)*dra for dyadic near/dra.  Odd pulses get
    small x offsets (no tie) so both branches appear in one aperture.
    """
    naz, nra = 64, 40
    near, dra, lam = 3550.0, 0.5, 0.031
    n = np.arange(naz) % 36
    tz = near + (n + 0.5) * dra
    tx = np.where(np.arange(naz) % 2 == 1, 0.75, 0.0)
    ty = np.zeros(naz)
    dim0, dim1 = 4, 2
    xx = np.zeros((dim0, dim1), order="F")
    yy = np.zeros((dim0, dim1), order="F")
    zz = np.zeros((dim0, dim1), order="F")
    xx[1, 0] = 0.125
    yy[2, 1] = -0.25
    index = np.asfortranarray(np.array([[10, 40], [20, 30], [32, 12], [50, 5]], dtype=np.int32))
    sint = np.asfortranarray(np.array([[16, 21], [30, 8], [62, 10], [20, 7]], dtype=np.int32))
    mask = np.ones((dim0, dim1), dtype=np.uint8, order="F")
    rng = np.random.default_rng(5)
    raw = np.asfortranarray((rng.standard_normal((nra, naz))
                             + 1j * rng.standard_normal((nra, naz))).astype(np.complex64))
    return dict(xxg1=xx, yyg1=yy, zzg1=zz, Mask=mask, Index=index, Sint=sint, wgsx=tx,
                wgsy=ty, wgsz=tz, RawData=raw, NearRange=np.float64(near),
                DeltaRange=np.float64(dra), Lambda=np.float64(lam))


INPUT_KEYS = ("xxg1", "yyg1", "zzg1", "Mask", "Index", "Sint", "wgsx", "wgsy", "wgsz",
              "RawData", "NearRange", "DeltaRange", "Lambda")


def main(argv):
    only = argv[argv.index("--only") + 1] if "--only" in argv else None
    ref = argv[argv.index("--reference") + 1] if "--reference" in argv else None
    mod = load_reference(ref)
    if only in (None, "small", "timing"):
        spec = synth.config_small()
        scene = synth.generate(spec)
        t = time.perf_counter()
        img = run_reference(mod, scene)
        seconds = time.perf_counter() - t
        print(f"small: reference took {seconds:.1f} s")
        if only != "timing":
            np.savez_compressed(HERE / "golden_small.npz", seed=spec.seed,
                                digest=synth.input_digest(scene), image=img)
        work = synth.nominal_pixel_pulses(scene)
        (HERE / "reference_timing.json").write_text(json.dumps({
            "workload": "small: DEM 256x64, 2001 pulses, Sint 400",
            "nominal_pixel_pulses": int(work), "seconds": round(seconds, 3),
            "gpix_pulse_per_s": work / seconds / 1e9, "cores": 1,
            "implementation": "reference FocalizzatoreBpPx (sar_focuser_puntual_noui.py:149), "
                              "unmodified, numba stub (plain NumPy)",
            "host": f"{platform.machine()} {platform.processor() or ''}".strip(),
            "numpy": np.__version__}, indent=1) + "\n")
    for name, make in (("edges", edges_scene), ("ties", ties_scene)):
        if only not in (None, name):
            continue
        scene = make()
        img = run_reference(mod, scene)
        np.savez_compressed(HERE / f"golden_{name}.npz", image=img,
                            **{k: scene[k] for k in INPUT_KEYS})
        print(f"{name}: {img.shape}, nonzero pixels {int(np.count_nonzero(img))}")


if __name__ == "__main__":
    main(sys.argv[1:])
