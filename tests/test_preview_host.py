"""Amplitude preview, host side: the PGM container and the no-fallback rule."""
import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import preview


def test_pgm_round_trip(tmp_path):
    a = np.arange(40 * 30, dtype=np.uint8).reshape(40, 30)
    p = preview.write_pgm(tmp_path / "a.pgm", a)
    assert p.read_bytes().startswith(b"P5\n30 40\n255\n")
    assert np.array_equal(preview.read_pgm(p), a)
    with pytest.raises(ValueError):
        preview.write_pgm(tmp_path / "b.pgm", a.reshape(-1))


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU error")
def test_no_cpu_fallback():
    with pytest.raises(RuntimeError, match="CUDA"):
        preview.amplitude_u8(np.ones((4, 5), dtype=np.complex128))
