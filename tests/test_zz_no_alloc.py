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


def test_noalloc_queue_that_does_not_fit_falls_back_to_one_cta_per_tile():
    """A staged=2 tuning on a scene whose chunk tables fit the built-in
    scratch but whose tile queue (62,500 tiles) does not: the call runs one
    CTA per tile instead and still gives the workspace entry point's image."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    dim0, dim1, naz, nra = 4000, 2000, 131072, 64
    dev = torch.device("cuda", 0)
    k = torch.arange(naz, dtype=torch.float64)
    tx, ty, tz = 0.5 * k, torch.full((naz,), -2000.0, dtype=torch.float64), \
        torch.full((naz,), 3000.0, dtype=torch.float64)
    xs = 16.0 * torch.arange(dim0, dtype=torch.float64) + 8.0
    ys = 100.0 + 0.01 * torch.arange(dim1, dtype=torch.float64)
    x = xs[:, None].expand(dim0, dim1)
    y = ys[None, :].expand(dim0, dim1)
    z = torch.zeros(dim0, dim1, dtype=torch.float64)
    near = float(torch.sqrt(torch.tensor(2100.0 ** 2 + 3000.0 ** 2))) - 4.0
    index = torch.round(x / 0.5).to(torch.int32)
    sint = torch.full((dim0, dim1), 7, dtype=torch.int32)
    mask = torch.ones(dim0, dim1, dtype=torch.uint8)
    g = torch.Generator().manual_seed(5)
    raw = torch.complex(torch.randn(naz, nra, generator=g),
                        torch.randn(naz, nra, generator=g)).to(torch.complex64).t()
    ds = scene_to_device(x.numpy(), y.numpy(), z.numpy(), mask.numpy(), index.numpy(),
                         tx.numpy(), ty.numpy(), tz.numpy(), raw, near, 0.5, 0.031,
                         sint.numpy(), device=dev)
    queued = dict(chunk=64, tile0=16, tile1=8, staged=2, window=128)
    ref = focus(ds, "mixed", tuning=dict(queued, staged=1), diagnostics=True).check()
    torch.cuda.synchronize()
    rc, out, nv, cs, ctr = _noalloc(ds, queued)
    _lib.check(rc)
    assert torch.equal(out, ref.image) and torch.equal(nv, ref.nvalid)
    assert torch.equal(cs, ref.checksum)
    assert int(nv.max().item()) > 0


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
