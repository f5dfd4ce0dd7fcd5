"""The allocation-free focusing entry point, called through the C ABI.

sarbp_focus_mixed_noalloc serves callers that cannot allocate device memory
(plugins in applications that own the device's memory pool, real-time
pipelines that may not call cudaMalloc, bindings without an allocator): its
scratch is a library-owned device array instead of a caller workspace.  Its
results must equal the workspace entry point's, on two calls in a row (the
array keeps the previous call's contents), within this suite's tolerances:
range-bin counts and checksums bit-exact, mixed-precision image quality bars.
This file is collected last so that a failure here never hides another test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import _lib, focus, quality, scene_to_device, synth

pytestmark = pytest.mark.gpu


def _scene(seed):
    spec = synth.SceneSpec(name=f"noalloc{seed}", seed=seed, dim0=64, dim1=32, x0=470.0,
                           naz=1201, sint_lo=300, sint_hi=360)
    return scene_to_device(*synth.focus_args(synth.generate(spec)), device="cuda:0")


def _noalloc(ds):
    lib = _lib.load()
    out = torch.empty((ds.npix, 2), dtype=torch.float64, device=ds.device)
    nv = torch.empty(ds.npix, dtype=torch.int32, device=ds.device)
    cs = torch.empty(ds.npix, dtype=torch.int64, device=ds.device)
    rc = lib.sarbp_focus_mixed_noalloc(C.byref(ds.struct()), None, out.data_ptr(),
                                       nv.data_ptr(), cs.data_ptr(), None,
                                       torch.cuda.current_stream(ds.device).cuda_stream)
    _lib.check(rc)
    torch.cuda.synchronize(ds.device)
    return out, nv, cs


def test_noalloc_matches_workspace_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    for seed in (21, 22):                     # two calls in a row, different scenes
        ds = _scene(seed)
        ref = focus(ds, "mixed", diagnostics=True)
        torch.cuda.synchronize()
        out, nv, cs = _noalloc(ds)
        assert torch.equal(nv, ref.nvalid)
        assert torch.equal(cs, ref.checksum)
        q = quality.compare(out.cpu().numpy(), ref.image.cpu().numpy())
        assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0 and q["rel_l2"] <= 1e-3, q


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
