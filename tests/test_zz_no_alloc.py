"""The allocation-free focusing entry point, called through the C ABI.

sarbp_focus_mixed_noalloc serves callers that cannot allocate device memory
(plugins in applications that own the device's memory pool, real-time
pipelines that may not call cudaMalloc, bindings without an allocator): its
scratch is a library-owned device array instead of a caller workspace.  Its
results must equal the workspace entry point's under the same tuning, bit
for bit (image, range-bin counts and checksums), on two calls in a row (the
array keeps the previous call's contents), with one CTA per tile and with
the persistent tile queue.  A bounded device wait that gives up must come
back from the call itself as SARBP_ETIMEOUT, since its caller holds no
workspace whose status it could read.  This file is collected last so that
a failure here never hides another test.
"""
import ctypes as C

import pytest
import torch

from sar_backprojection_gb300 import _lib, focus, scene_to_device, synth
from sar_backprojection_gb300.focuser import resolve_tuning

pytestmark = pytest.mark.gpu


def _scene(seed):
    spec = synth.SceneSpec(name=f"noalloc{seed}", seed=seed, dim0=64, dim1=32, x0=470.0,
                           naz=1201, sint_lo=300, sint_hi=360)
    return scene_to_device(*synth.focus_args(synth.generate(spec)), device="cuda:0")


def _noalloc(ds, tuning=None):
    lib = _lib.load()
    out = torch.empty((ds.npix, 2), dtype=torch.float64, device=ds.device)
    nv = torch.empty(ds.npix, dtype=torch.int32, device=ds.device)
    cs = torch.empty(ds.npix, dtype=torch.int64, device=ds.device)
    ctr = torch.zeros(_lib.NUM_COUNTERS, dtype=torch.int64, device=ds.device)
    t = C.byref(resolve_tuning(tuning)) if tuning is not None else None
    rc = lib.sarbp_focus_mixed_noalloc(C.byref(ds.struct()), t, out.data_ptr(),
                                       nv.data_ptr(), cs.data_ptr(), ctr.data_ptr(),
                                       torch.cuda.current_stream(ds.device).cuda_stream)
    torch.cuda.synchronize(ds.device)
    return rc, out, nv, cs, ctr


@pytest.mark.parametrize("tuning", [None, dict(chunk=32, tile0=16, tile1=8, staged=2,
                                               window=128)],
                         ids=["default", "queue"])
def test_noalloc_matches_workspace_entry_point_twice(tuning):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    for seed in (21, 22):                     # two calls in a row, different scenes
        ds = _scene(seed)
        ref = focus(ds, "mixed", tuning=tuning, diagnostics=True).check()
        torch.cuda.synchronize()
        rc, out, nv, cs, ctr = _noalloc(ds, tuning)
        _lib.check(rc)
        assert torch.equal(out, ref.image)
        assert torch.equal(nv, ref.nvalid)
        assert torch.equal(cs, ref.checksum)
        assert int(ctr[_lib.CTR_TIMEOUTS].item()) == 0


def test_noalloc_reports_a_wait_that_runs_out():
    """withhold=1 leaves one stage copy of every pass unissued, so its bounded
    wait gives up: the call returns SARBP_ETIMEOUT, and the next call on the
    same context is bit-identical to the workspace entry point again."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    ds = _scene(24)
    bad = dict(chunk=64, tile0=16, tile1=16, staged=1, window=160, wait_polls=64, withhold=1)
    rc, _, _, _, ctr = _noalloc(ds, bad)
    assert rc == _lib.SARBP_ETIMEOUT
    assert "gave up" in _lib.last_error()
    assert int(ctr[_lib.CTR_TIMEOUTS].item()) > 0
    good = dict(bad, withhold=0, wait_polls=0)
    rc, out, nv, _, ctr = _noalloc(ds, good)
    _lib.check(rc)
    ref = focus(ds, "mixed", tuning=good, diagnostics=True).check()
    torch.cuda.synchronize()
    assert torch.equal(out, ref.image) and torch.equal(nv, ref.nvalid)
    assert int(ctr[_lib.CTR_TIMEOUTS].item()) == 0


def test_noalloc_rejects_scenes_beyond_its_limit():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    ds = _scene(23)
    s = _lib.Scene.from_buffer_copy(ds.struct())
    s.naz = 131072 + 1                         # rejected before any device work
    out = torch.empty((ds.npix, 2), dtype=torch.float64, device=ds.device)
    rc = lib.sarbp_focus_mixed_noalloc(C.byref(s), None, out.data_ptr(), None, None, None,
                                       torch.cuda.current_stream(ds.device).cuda_stream)
    assert rc == _lib.SARBP_ERANGE
    assert "131072" in _lib.last_error()
