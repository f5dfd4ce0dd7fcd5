"""Amplitude preview of a focused image, computed on the GPU.

The reference's visualiser scales |image| to 8 bits with the maximum at
15 x the mean amplitude and clips (img_visualizer.py:23-46,
`np.clip(|x| * 255 / (15*mean|x|), 0, 255).astype(uint8)`), then writes a PNG
with PIL.  Neither PIL nor matplotlib is part of this package's runtime, so
the 8-bit image is written as a binary PGM (P5) -- a headless buffer any
image tool reads.  ``astype(uint8)`` truncates, as NumPy's cast does.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch


def amplitude_u8(image, scale_factor: float = 15.0, device=None) -> torch.Tensor:
    """8-bit amplitude of a complex image (tensor or array), on the device.

    ``image`` may be complex (any shape) or float pairs (..., 2).  Returns a
    uint8 tensor of the image's shape (rows = first axis).
    """
    if not isinstance(image, torch.Tensor):
        image = torch.from_numpy(np.ascontiguousarray(image))
    if device is not None or image.device.type == "cpu":
        dev = torch.device(device) if device is not None else (
            torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
        image = image.to(dev)
    if not torch.is_complex(image):
        image = torch.view_as_complex(image.to(torch.float64).contiguous())
    mag = image.abs().to(torch.float64)
    mean = mag.mean()
    max_val = scale_factor * mean
    scaled = torch.where(max_val > 0, mag * (255.0 / max_val), torch.zeros_like(mag))
    return torch.clamp(scaled, 0.0, 255.0).to(torch.uint8)


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
    return write_pgm(path, amplitude_u8(image, scale_factor))
