"""Amplitude preview: the reference visualiser's 15*mean scaling, PGM output."""
import numpy as np

from sar_backprojection_gb300 import preview


def test_matches_reference_scaling(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.standard_normal((40, 30)) + 1j * rng.standard_normal((40, 30))
    img[3, 4] = 1000.0                                      # a bright target clips
    u8 = preview.amplitude_u8(img, device="cpu").numpy()
    mag = np.abs(img)
    ref = np.clip(mag * (255.0 / (15 * np.mean(mag))), 0, 255).astype(np.uint8)
    assert np.array_equal(u8, ref)
    p = preview.write_pgm(tmp_path / "a.pgm", u8)
    assert np.array_equal(preview.read_pgm(p), ref)
    pairs = np.stack([img.real, img.imag], axis=-1)
    assert np.array_equal(preview.amplitude_u8(pairs, device="cpu").numpy(), ref)


def test_all_zero_image():
    u8 = preview.amplitude_u8(np.zeros((4, 5), dtype=np.complex128), device="cpu")
    assert int(u8.max()) == 0
