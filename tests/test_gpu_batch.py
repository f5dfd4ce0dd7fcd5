"""Batched persistent focusing: each scene's result equals its single-scene result.

The batch kernel runs the same per-tile code as the single-scene staged
kernel, so images, contributor counts and range-bin checksums must be
bit-identical, in a direct launch and in CUDA-graph replays; and every scene
must meet the mixed-precision bars against the FP64 kernel.
"""
import pytest
import torch

from sar_backprojection_gb300 import batch, focus, quality, scene_to_device, synth

pytestmark = pytest.mark.gpu

SIZES = [(128, 32, 2001, 200, 260), (300, 48, 3001, 400, 600), (96, 40, 2401, 900, 1300),
         (200, 64, 4001, 1200, 1800), (64, 32, 2001, 300, 400)]


@pytest.fixture(scope="module")
def scenes():
    out = []
    for i, (d0, d1, naz, s_lo, s_hi) in enumerate(SIZES):
        spec = synth.scaled_full(100 + i, d0, d1, naz, s_lo, s_hi)
        sc = synth.generate(spec, raw_device="cuda")
        out.append(scene_to_device(*synth.focus_args(sc), device="cuda"))
    return out


@pytest.mark.parametrize("tiling", batch.STAGED_TILINGS,
                         ids=lambda t: f"{t[0]}x{t[1]}w{t[2]}c{t[3]}")
@pytest.mark.parametrize("graph", [False, True], ids=["direct", "graph"])
def test_batch_equals_single_scene(scenes, tiling, graph):
    tuning = batch.staged_tuning(*tiling)
    bf = batch.BatchFocuser(scenes, tuning, diagnostics=True, graph=graph)
    for _ in range(2):                        # a second replay must not change anything
        bf.run()
    torch.cuda.synchronize()
    assert int(bf.counters[3].item()) == 0    # no bounded wait gave up
    for sl in bf.slots:
        ref = focus(sl.scene, "mixed", tuning=tuning, diagnostics=True)
        torch.cuda.synchronize()
        assert torch.equal(sl.out, ref.image)
        assert torch.equal(sl.nvalid, ref.nvalid)
        assert torch.equal(sl.checksum, ref.checksum)


def test_batch_quality_against_fp64(scenes):
    bf = batch.BatchFocuser(scenes, graph=True)
    bf.run()
    torch.cuda.synchronize()
    for sl, img in zip(bf.slots, bf.images()):
        ref = focus(sl.scene, "fp64")
        torch.cuda.synchronize()
        q = quality.compare(torch.view_as_real(img.t().reshape(-1)).cpu().numpy(),
                            ref.image.cpu().numpy())
        assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0, q


def test_autotuner_picks_a_candidate(scenes):
    at = batch.Autotuner(repeats=1)
    t = at.pick(scenes[:3])
    assert (t.tile0, t.tile1, t.window, t.chunk) in batch.STAGED_TILINGS and t.staged == 1
    assert at.pick(scenes[:3]).tile0 == t.tile0        # cached
    assert len(at.timings) == 1


def test_uneven_48_scene_batch():
    """The batch the bench times: the 48 uneven scenes (DEM 128x32..2000x250,
    2001..20001 pulses, Sint 200..1800), the tiling the autotuner picks for
    them, one graph-captured persistent launch without checksum outputs.
    Every scene's image must equal its single-scene launch of the same tuning
    bit for bit and meet the mixed-precision bars against the FP64 kernel
    (whose range bins and values are pinned to the oracle elsewhere)."""
    specs = synth.uneven_specs(48)
    scenes = [scene_to_device(*synth.focus_args(synth.generate(sp, raw_device="cuda")),
                              device="cuda") for sp in specs]
    tuning = batch.Autotuner(repeats=1).pick(scenes)
    bf = batch.BatchFocuser(scenes, tuning, graph=True)
    for _ in range(2):
        bf.run()
    torch.cuda.synchronize()
    for sl, img in zip(bf.slots, bf.images()):
        single = focus(sl.scene, "mixed", tuning=tuning).check()
        torch.cuda.synchronize()
        assert torch.equal(sl.out, single.image)
        ref = focus(sl.scene, "fp64")
        torch.cuda.synchronize()
        q = quality.compare(torch.view_as_real(img.t().reshape(-1)).cpu().numpy(),
                            ref.image.cpu().numpy())
        assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0 and q["rel_l2"] <= 1e-3, q
