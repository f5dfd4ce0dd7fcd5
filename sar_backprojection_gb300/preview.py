"""Amplitude preview of a focused image, computed on the GPU.

The reference's visualiser scales |image| to 8 bits with the maximum at
15 x the mean amplitude and clips (img_visualizer.py:23-46,
`np.clip(|x| * (255 / (15*mean|x|)), 0, 255).astype(uint8)`), then writes a
PNG with PIL.  Here the scaling runs in libsarbp's kernels
(``sarbp_amplitude_u8``: fixed-order mean, FP64 hypot and scale, truncating
cast), and the 8-bit image is written as a binary PGM (P5) -- a headless
buffer any image tool reads; PIL and matplotlib are not part of this
package's runtime.

Orientation: the visualiser reads ``SlcMatr_real.dat`` as a (D1, D0) C-order
array, i.e. the column-major (D0, D1) image with range lines as rows;
``save_preview`` writes the PGM the same way (D1 rows of D0 pixels).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import torch

from . import _lib


def _device_pairs(image, device) -> tuple[torch.Tensor, tuple, str]:
    """(npix, 2) float64 device tensor of the image's pixels in memory order,
    the image's shape and that order ("F" or "C")."""
    if isinstance(image, torch.Tensor):
        t = image
        if torch.is_complex(t):
            shape = tuple(t.shape)
            t = torch.view_as_real(t.to(torch.complex128).contiguous())
        else:
            shape = tuple(t.shape[:-1])
            t = t.to(torch.float64).contiguous()
        order = "C"
    else:
        a = np.asarray(image)
        if a.dtype.kind == "c":
            shape = a.shape
            order = "F" if (a.ndim > 1 and a.flags.f_contiguous) else "C"
            a = np.asarray(a.reshape(-1, order=order), dtype=np.complex128)
            t = torch.from_numpy(np.ascontiguousarray(a).view(np.float64).reshape(-1, 2))
        else:
            shape = a.shape[:-1]
            order = "C"
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 2))
    if not torch.cuda.is_available():
        raise RuntimeError("the amplitude preview runs on a CUDA device (no CPU fallback)")
    dev = torch.device(device) if device is not None else (
        t.device if t.device.type == "cuda" else torch.device("cuda", torch.cuda.current_device()))
    return t.reshape(-1, 2).to(dev).contiguous(), shape, order


def amplitude_u8(image, scale_factor: float = 15.0, device=None,
                 return_mean: bool = False):
    """8-bit amplitude of a complex image, on the device.

    ``image``: complex (any shape; NumPy or torch) or float pairs (..., 2).
    Returns a uint8 device tensor of the image's shape (same indexing), and
    with ``return_mean`` also the mean amplitude the scale used.
    """
    pairs, shape, order = _device_pairs(image, device)
    npix = pairs.shape[0]
    dev = pairs.device
    out = torch.empty(npix, dtype=torch.uint8, device=dev)
    mean = torch.empty(1, dtype=torch.float64, device=dev)
    scratch = torch.empty(_lib.PREVIEW_SCRATCH_BYTES // 8, dtype=torch.float64, device=dev)
    if npix:
        _lib.check(_lib.load().sarbp_amplitude_u8(
            pairs.data_ptr(), npix, C.c_double(scale_factor), out.data_ptr(), mean.data_ptr(),
            scratch.data_ptr(), _lib.PREVIEW_SCRATCH_BYTES,
            torch.cuda.current_stream(dev).cuda_stream))
    if order == "F":
        u8 = out.reshape(tuple(reversed(shape))).permute(*reversed(range(len(shape))))
    else:
        u8 = out.reshape(shape)
    return (u8, float(mean.item())) if return_mean else u8


def write_pgm(path, u8) -> Path:
    """Write a 2-D uint8 array/tensor as a binary PGM (rows = first axis)."""
    a = u8.cpu().numpy() if isinstance(u8, torch.Tensor) else np.asarray(u8, dtype=np.uint8)
    if a.ndim != 2:
        raise ValueError("a preview is a 2-D image")
    p = Path(path)
    with open(p, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(np.ascontiguousarray(a, dtype=np.uint8).tobytes())
    return p


def read_pgm(path) -> np.ndarray:
    data = Path(path).read_bytes()
    parts = data.split(b"\n", 3)
    if parts[0] != b"P5":
        raise ValueError(f"{path}: not a binary PGM")
    w, h = (int(v) for v in parts[1].split())
    return np.frombuffer(parts[3], dtype=np.uint8, count=w * h).reshape(h, w)


def save_preview(image, path, scale_factor: float = 15.0) -> Path:
    """PGM of a (D0, D1) image in the reference visualiser's orientation:
    D1 rows (range) of D0 pixels (azimuth)."""
    return write_pgm(path, amplitude_u8(image, scale_factor).T)
