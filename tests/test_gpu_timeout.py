"""Bounded device waits: a wait that runs out is reported and the context survives.

The staged kernels bound every mbarrier wait.  The diagnostic tuning field
``withhold=1`` never issues the first stage copy of each pass, so that
stage's wait runs out after ``wait_polls`` polls: the CTAs stop, let the
copies they did issue land, and mark the workspace status.  The test checks
the reported status, the timeout counter, that the status is cleared once
read, that the drop-in call raises, and that the next normal call on the
same context gives the same image as before.
"""
import pytest
import torch

from sar_backprojection_gb300 import FocalizzatoreBpPx, _lib, focus, scene_to_device, synth

pytestmark = pytest.mark.gpu

WITHHOLD = dict(chunk=64, tile0=16, tile1=16, staged=1, window=160, wait_polls=64, withhold=1)


@pytest.fixture(scope="module")
def scene():
    spec = synth.scaled_full(31, 256, 64, 4001, 600, 900)
    sc = synth.generate(spec, raw_device="cuda")
    return sc, scene_to_device(*synth.focus_args(sc), device="cuda")


@pytest.mark.parametrize("staged", [1, 2], ids=["per_tile", "queue"])
def test_wait_that_runs_out_is_reported(scene, staged):
    _, ds = scene
    good = focus(ds, "mixed", tuning=dict(WITHHOLD, withhold=0, staged=staged),
                 diagnostics=True).check()
    torch.cuda.synchronize()
    bad = focus(ds, "mixed", tuning=dict(WITHHOLD, staged=staged), diagnostics=True)
    assert bad.status() == _lib.SARBP_ETIMEOUT
    assert "gave up" in _lib.last_error()
    assert int(bad.counters[_lib.CTR_TIMEOUTS].item()) > 0
    assert bad.status() == _lib.SARBP_OK          # cleared once read
    again = focus(ds, "mixed", tuning=dict(WITHHOLD, withhold=0, staged=staged),
                  diagnostics=True).check()
    torch.cuda.synchronize()
    assert int(again.counters[_lib.CTR_TIMEOUTS].item()) == 0
    assert torch.equal(again.image, good.image)
    assert torch.equal(again.nvalid, good.nvalid)


def test_drop_in_call_raises_on_timeout(scene):
    sc, _ = scene
    with pytest.raises(_lib.SarbpError) as e:
        FocalizzatoreBpPx(*synth.focus_args(sc), precision="mixed", tuning=WITHHOLD)
    assert e.value.status == _lib.SARBP_ETIMEOUT
    img = FocalizzatoreBpPx(*synth.focus_args(sc), precision="mixed",
                            tuning=dict(WITHHOLD, withhold=0))
    assert img.shape == (256, 64)
