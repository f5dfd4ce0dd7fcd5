"""TEST INFRASTRUCTURE ONLY -- the oracle the focuser is checked against.

ctypes wrapper of ``bp_oracle.c``, the CPU FP64 restatement of the reference's
``process_point`` / ``FocalizzatoreBpPx`` (sar_focuser_puntual_noui.py:9-284).
Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference legs may import this module; the focusing product never does.

The restatement is pinned against the reference itself: tests/golden/ holds
outputs of the unmodified reference ``FocalizzatoreBpPx`` run in NumPy (the
generating script is tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import shutil
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "bp_oracle.c"
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "libsarbp_oracle.so"
CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
          "-fvisibility=hidden", "-std=c11"]
_ELF = {"x86_64": 62, "aarch64": 183, "arm64": 183}
_lock = threading.Lock()
_lib = None


def _elf_machine(p: Path):
    try:
        hdr = p.read_bytes()[:20]
    except OSError:
        return None
    return int.from_bytes(hdr[18:20], "little") if hdr[:4] == b"\x7fELF" else None


def build(force: bool = False) -> Path:
    """Compile bp_oracle.c with gcc (-ffp-contract=off: no fused multiply-add)."""
    if (not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime
            and _elf_machine(LIB) == _ELF.get(platform.machine())):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([cc, *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    with _lock:
        if _lib is None:
            lib = C.CDLL(str(build()))
            P = C.c_void_p
            lib.sarbp_oracle_focus.restype = C.c_int
            lib.sarbp_oracle_focus.argtypes = [P, P, P, P, P, P, P, P, P, P,
                                               C.c_int64, C.c_int64, C.c_int64,
                                               C.c_double, C.c_double, C.c_double,
                                               P, C.c_int64, P, P, P, C.c_int]
            lib.sarbp_oracle_mix64.restype = C.c_uint64
            lib.sarbp_oracle_mix64.argtypes = [C.c_int64, C.c_int64]
            lib.sarbp_oracle_max_threads.restype = C.c_int
            _lib = lib
    return _lib


def max_threads() -> int:
    return int(load().sarbp_oracle_max_threads())


def mix64(pulse: int, rbin: int) -> int:
    return int(load().sarbp_oracle_mix64(pulse, rbin))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _flat_f(a, dtype):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    a = np.asarray(a)
    return np.ascontiguousarray(a.astype(dtype, copy=False).reshape(-1, order="F"))


def _raw_pulse_major(raw) -> tuple[np.ndarray, int, int]:
    """(Nra, Naz) complex64 -> contiguous pulse-major float32 pairs."""
    if hasattr(raw, "detach"):
        import torch
        t = raw.detach()
        if t.device.type != "cpu":
            t = t.cpu()
        nra, naz = t.shape
        arr = t.t().contiguous().numpy()            # (naz, nra) complex64
    else:
        r = np.asarray(raw)
        if r.dtype != np.complex64:
            r = r.astype(np.complex64)
        nra, naz = r.shape
        arr = np.ascontiguousarray(r.T)
    return arr.view(np.float32).reshape(-1), int(nra), int(naz)


def focus(xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, Raw_Data, near_range, dra,
          lambda_val, Sint, *, pixels=None, nthreads: int = 0, raw_prepared=None):
    """Oracle focusing with the reference's argument order.

    Returns (values complex128, nvalid int32, checksum uint64): the full
    (dim0, dim1) column-major image when ``pixels`` is None, else 1-D arrays
    for the listed column-major pixel indices.  ``raw_prepared`` may pass a
    (flat float32 pulse-major, nra, naz) triple to skip the raw re-layout.
    """
    lib = load()
    dim0, dim1 = (int(v) for v in np.shape(xxg1))
    x, y, z = (_flat_f(a, np.float64) for a in (xxg1, yyg1, zzg1))
    m = _flat_f(mask, np.uint8)
    idx = _flat_f(index, np.int32)
    s = _flat_f(Sint, np.int32)
    m = np.where(s == -9999, np.uint8(0), m)                   # :195-198
    wx, wy, wz = (np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1))
                  for w in (wgsx, wgsy, wgsz))
    raw, nra, naz = raw_prepared if raw_prepared is not None else _raw_pulse_major(Raw_Data)
    if pixels is None:
        count = dim0 * dim1
        pix = None
    else:
        pix = np.ascontiguousarray(np.asarray(pixels, dtype=np.int64))
        count = int(pix.size)
    out = np.zeros(2 * count, dtype=np.float64)
    nv = np.zeros(count, dtype=np.int32)
    cs = np.zeros(count, dtype=np.uint64)
    rc = lib.sarbp_oracle_focus(_ptr(x), _ptr(y), _ptr(z), _ptr(m), _ptr(idx), _ptr(s),
                                _ptr(wx), _ptr(wy), _ptr(wz), _ptr(raw), nra, naz, nra,
                                float(near_range), float(dra), float(lambda_val),
                                _ptr(pix) if pix is not None else None, count,
                                _ptr(out), _ptr(nv), _ptr(cs), int(nthreads))
    if rc != 0:
        raise ValueError("oracle rejected its arguments")
    vals = out.view(np.complex128)
    if pixels is None:
        return (np.reshape(vals, (dim0, dim1), order="F"),
                np.reshape(nv, (dim0, dim1), order="F"),
                np.reshape(cs, (dim0, dim1), order="F"))
    return vals, nv, cs


def focus_scene(scene: dict, **kw):
    """``focus`` on a synth-style scene dict."""
    return focus(scene["xxg1"], scene["yyg1"], scene["zzg1"], scene["Mask"], scene["Index"],
                 scene["wgsx"], scene["wgsy"], scene["wgsz"], scene["RawData"],
                 scene["NearRange"], scene["DeltaRange"], scene["Lambda"], scene["Sint"], **kw)
