"""The C serving queue: every job's image equals its single-scene image."""
import pytest
import torch

from sar_backprojection_gb300 import focus, scene_to_device, synth
from sar_backprojection_gb300.serve import NativeQueue

pytestmark = pytest.mark.gpu

SIZES = [(128, 32, 2001, 200, 260), (300, 48, 3001, 400, 600), (96, 40, 2401, 900, 1300),
         (200, 64, 4001, 1200, 1800), (64, 32, 2001, 300, 400), (160, 24, 2501, 500, 700)]


@pytest.fixture(scope="module")
def scenes():
    out = []
    for i, (d0, d1, naz, s_lo, s_hi) in enumerate(SIZES):
        spec = synth.scaled_full(300 + i, d0, d1, naz, s_lo, s_hi)
        sc = synth.generate(spec, raw_device="cuda")
        out.append(scene_to_device(*synth.focus_args(sc), device="cuda"))
    return out


@pytest.mark.parametrize("slots", [2, 8], ids=["2slots", "8slots"])
def test_queue_jobs_equal_single_scene(scenes, slots):
    with NativeQueue(max_slots=slots, wave_items=200) as q:
        jobs = [q.submit(ds) for ds in scenes * 2]          # more jobs than slots
        imgs = [q.wait(j) for j in jobs]
    for ds, img in zip(scenes * 2, imgs):
        ref = focus(ds, "mixed", tuning=q.tuning).check()
        torch.cuda.synchronize()
        assert torch.equal(img, ref.image)


def test_queue_poll_reports_once(scenes):
    with NativeQueue(max_slots=4) as q:
        j = q.submit(scenes[0])
        q.wait(j)
        with pytest.raises(Exception):
            q.poll(j)                                     # id released after completion


def test_queue_cancels_a_waiting_job(scenes):
    """With one scene slot, a job behind two others is still waiting when it
    is cancelled: it reports SARBP_ECANCELED and the others still finish."""
    from sar_backprojection_gb300 import _lib
    with NativeQueue(max_slots=1) as q:
        a = q.submit(scenes[3])                  # the largest scene first
        b = q.submit(scenes[0])
        c = q.submit(scenes[1])
        q.cancel(c)
        with pytest.raises(_lib.SarbpError) as e:
            q.wait(c)
        assert e.value.status == _lib.SARBP_ECANCELED
        for j, ds in ((a, scenes[3]), (b, scenes[0])):
            img = q.wait(j)
            ref = focus(ds, "mixed", tuning=q.tuning).check()
            torch.cuda.synchronize()
            assert torch.equal(img, ref.image)
        with pytest.raises(_lib.SarbpError):
            q.cancel(a)                           # done and released
