"""Amplitude preview on the GPU against the reference visualiser's scaling.

img_visualizer.py:23-46: np.clip(|x| * (255 / (15 * mean|x|)), 0, 255)
.astype(uint8).  The kernel's mean sums in a fixed order of its own, so the
NumPy scaling is evaluated with the mean the kernel reports (which must equal
np.mean to 1e-13 relative); every byte must then match except where the
scaled amplitude lies within 1e-9 of an integer (a last-bit difference of
hypot could truncate the other way there).
"""
import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import preview

pytestmark = pytest.mark.gpu


def _reference_bytes(img, mean, scale=15.0):
    mag = np.abs(img)
    x = mag * (255.0 / (scale * mean))
    return np.clip(x, 0, 255).astype(np.uint8), x


@pytest.mark.parametrize("shape,order", [((400, 250), "F"), ((123, 77), "C"), ((1, 5), "F")])
def test_matches_reference_scaling(shape, order):
    rng = np.random.default_rng(0)
    img = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    img.flat[3] = 1000.0                                   # a bright target clips
    img = np.asfortranarray(img) if order == "F" else np.ascontiguousarray(img)
    u8, mean = preview.amplitude_u8(img, return_mean=True)
    u8 = u8.cpu().numpy()
    assert u8.shape == shape
    assert mean == pytest.approx(np.mean(np.abs(img)), rel=1e-13)
    ref, x = _reference_bytes(img, mean)
    near = np.abs(x - np.rint(x)) < 1e-9
    assert np.array_equal(u8[~near], ref[~near])
    assert int(u8.max()) == int(ref.max())


def test_device_image_pairs_and_zero_image(tmp_path):
    img = torch.randn(64, 32, dtype=torch.complex128, device="cuda")
    pairs = torch.view_as_real(img)
    a = preview.amplitude_u8(img)
    b = preview.amplitude_u8(pairs)
    assert torch.equal(a, b)
    z = preview.amplitude_u8(np.zeros((4, 5), dtype=np.complex128))
    assert int(z.max()) == 0
    p = preview.save_preview(img.cpu().numpy(), tmp_path / "p.pgm")
    assert preview.read_pgm(p).shape == (32, 64)          # range lines as rows
