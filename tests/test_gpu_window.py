"""The staged kernels' fast path trusts each stage's range window.

A stage runs on the fast path only when the window prologue's bound says
every bin the warp's pixels can reach lies inside the staged window; the
fast path then reads shared memory without a per-pulse window test (an
out-of-window column would be clamped to the window's edge).  The bound is
conservative by construction (segment endpoint and closest-point distances,
the stage's chord deviation, approximate square roots inside a one-bin
margin); this test attacks it with geometry that stresses every term: steep
rough terrain (80 m relief at 40 m correlation), +-1 m low-frequency motion
of the platform, short apertures at the swath edges, and windows from 128
bins (too narrow for many tiles: their stages take the generic path) to 208.
Range-bin selection must equal the oracle's bit for bit: a clamped read
would change the per-pixel (pulse, bin) checksum.
"""
from dataclasses import replace

import numpy as np
import pytest
import torch

from oracle import oracle
from sar_backprojection_gb300 import focus, quality, scene_to_device, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rough():
    spec = replace(synth.config_full(41), name="rough", dim0=320, dim1=96,
                         az_spacing=5.0, x0=400.0, naz=4801, terrain_sigma=80.0,
                         terrain_corr=40.0, motion_amp=1.0, sint_lo=200, sint_hi=1800,
                         n_targets=40)
    sc = synth.generate(spec, raw_device="cuda")
    host = dict(sc)
    host["RawData"] = sc["RawData"].cpu()
    return sc, oracle.focus_scene(host)


@pytest.mark.parametrize("tuning", [
    dict(chunk=128, tile0=16, tile1=16, staged=1, window=128),
    dict(chunk=128, tile0=16, tile1=16, staged=1, window=160),
    dict(chunk=128, tile0=16, tile1=16, staged=1, window=208),
    dict(chunk=64, tile0=16, tile1=8, staged=1, window=128),
    dict(chunk=32, tile0=64, tile1=4, staged=1, window=128),
], ids=["16x16w128", "16x16w160", "16x16w208", "16x8w128", "64x4w128"])
def test_rough_terrain_bins_match_the_oracle(rough, tuning):
    sc, (oimg, onv, ocs) = rough
    ds = scene_to_device(*synth.focus_args(sc), device="cuda")
    res = focus(ds, "mixed", tuning=tuning, diagnostics=True).check()
    torch.cuda.synchronize()
    shape = (ds.dim0, ds.dim1)
    nv = res.nvalid.cpu().numpy().reshape(shape, order="F")
    cs = res.checksum.cpu().numpy().view(np.uint64).reshape(shape, order="F")
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    q = quality.compare(res.to_numpy(*shape), oimg)
    assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0, q
    print(tuning, "window misses served from L2:", int(res.counters[1].item()))
