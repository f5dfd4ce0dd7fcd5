"""One scene split by azimuth block: each block focused from its own raw
window (re-based pulse indices) gives the whole scene's image bit for bit.

The blocks run one after another on one device here (each is an ordinary
focusing call; nothing waits on another block), as the ranks of a multi-GPU
split would run them side by side.  Both kernels are checked: FP64 (whose
result depends on nothing but the pixel) and mixed precision, whose chunk
references and pulse tables match the whole scene's because every window
starts on a multiple of the longest chunk.
"""
import numpy as np
import pytest

from sar_backprojection_gb300 import FocalizzatoreBpPx, partition, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    spec = synth.scaled_full(81, 512, 64, 8001, 600, 1000)
    sc = synth.azimuth_columns(synth.generate(spec, raw_device="cuda"))
    sc["RawData"] = sc["RawData"].cpu().numpy()            # (nra, naz), column-major bytes
    return sc


@pytest.mark.parametrize("precision,tuning", [
    ("fp64", None),
    ("mixed", dict(chunk=128, tile0=16, tile1=16, staged=1, window=208)),
    ("mixed", dict(chunk=64, tile0=16, tile1=16, staged=1, window=208)),
    ("mixed", dict(chunk=32, tile0=32, tile1=8, staged=0)),
], ids=["fp64", "c128", "c64", "c32_l1"])
@pytest.mark.parametrize("nranks", [2, 4])
def test_blocks_equal_the_single_call(scene, precision, tuning, nranks):
    args = synth.focus_args(scene)
    whole = FocalizzatoreBpPx(*args, precision=precision, tuning=tuning)
    blocks = partition.plan(scene["Index"], scene["Sint"], scene["Mask"],
                            scene["RawData"].shape[1], nranks, axis=1)
    assert all(b.pulses < scene["RawData"].shape[1] for b in blocks if b.lines)
    imgs = [partition.focus_block(args, blocks, r, precision=precision, tuning=tuning)
            for r in range(nranks)]
    got = partition.assemble(blocks, imgs, whole.shape)
    assert np.array_equal(np.ascontiguousarray(got).view(np.uint64),
                          np.ascontiguousarray(whole).view(np.uint64))
