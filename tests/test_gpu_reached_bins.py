"""Reached-bins upload: only the range bins some aperture can reach are copied.

The bound (sarbp_raw_bin_range) must contain every bin any kernel reads.  The
test uploads a scene that way, then poisons every other bin of the device
raw buffer with NaN: an image equal bit for bit to the full-upload image
(and free of NaN) shows the kernels never read outside the bound.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden_scene
from sar_backprojection_gb300 import FocalizzatoreBpPx, focus, scene_to_device, synth
from sar_backprojection_gb300 import focuser

pytestmark = pytest.mark.gpu


def _host_args(sc):
    args = list(synth.focus_args(sc))
    raw = args[8]
    if isinstance(raw, torch.Tensor):
        raw = raw.cpu()
    args[8] = np.asfortranarray(np.asarray(raw, dtype=np.complex64))
    return args


def _poison(ds):
    torch.cuda.synchronize()
    if ds.bin_lo > 0:
        ds.raw[:, : ds.bin_lo, :] = float("nan")
    ds.raw[:, ds.bin_hi + 1:, :] = float("nan")


SCENES = {
    "uneven": lambda: synth.generate(synth.scaled_full(41, 300, 48, 3001, 400, 700),
                                     raw_device="cuda"),
    "small": lambda: synth.generate(synth.config_small(3)),
}


@pytest.mark.parametrize("name", sorted(SCENES))
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_reached_bins_are_all_that_is_read(name, precision):
    args = _host_args(SCENES[name]())
    full = scene_to_device(*args, device="cuda")
    part = scene_to_device(*args, device="cuda", raw_bins="reached")
    assert 0 <= part.bin_lo <= part.bin_hi <= part.nra - 1
    assert part.h2d_bytes < full.h2d_bytes
    _poison(part)
    a = focus(full, precision, diagnostics=True)
    b = focus(part, precision, diagnostics=True)
    torch.cuda.synchronize()
    assert not torch.isnan(b.image).any()
    assert torch.equal(a.image, b.image)
    assert torch.equal(a.nvalid, b.nvalid) and torch.equal(a.checksum, b.checksum)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_reached_bins_on_the_edge_cases(precision):
    """Golden edge scene: bins across 0 and Nra-2..Nra, masks, odd Sint."""
    sc, _ = load_golden_scene("edges")
    args = list(sc[k] for k in ("xxg1", "yyg1", "zzg1", "Mask", "Index", "wgsx", "wgsy",
                                "wgsz", "RawData", "NearRange", "DeltaRange", "Lambda", "Sint"))
    args[8] = np.asfortranarray(np.asarray(args[8], dtype=np.complex64))
    full = scene_to_device(*args, device="cuda")
    part = scene_to_device(*args, device="cuda", raw_bins="reached")
    _poison(part)
    a = focus(full, precision, diagnostics=True)
    b = focus(part, precision, diagnostics=True)
    torch.cuda.synchronize()
    assert torch.equal(a.image, b.image)
    assert torch.equal(a.nvalid, b.nvalid) and torch.equal(a.checksum, b.checksum)


def test_drop_in_call_reports_bytes_moved():
    args = _host_args(SCENES["uneven"]())
    img = FocalizzatoreBpPx(*args, precision="mixed")
    lo, hi = focuser.last_call["raw_bins"]
    nra, naz = args[8].shape
    assert focuser.last_call["h2d_bytes"] < nra * naz * 8
    assert 0 <= lo <= hi < nra and img.shape == args[0].shape


@pytest.mark.parametrize("name", sorted(SCENES))
def test_streamed_drop_in_equals_resident_focus(name):
    """The streamed drop-in call (pulse-block uploads overlapped by queue
    segments) gives the resident scene's image bit for bit."""
    args = _host_args(SCENES[name]())
    full = scene_to_device(*args, device="cuda")
    ref = focus(full, "mixed").check().to_numpy(full.dim0, full.dim1)
    img = FocalizzatoreBpPx(*args, precision="mixed")
    assert focuser.last_call["streamed"]
    assert np.array_equal(np.ascontiguousarray(img).view(np.uint64),
                          np.ascontiguousarray(ref).view(np.uint64))
    img1 = FocalizzatoreBpPx(*args, precision="mixed",
                             tuning=dict(chunk=128, tile0=16, tile1=8, staged=1, window=128))
    ref1 = focus(full, "mixed", tuning=dict(chunk=128, tile0=16, tile1=8, staged=1,
                                            window=128)).check().to_numpy(full.dim0, full.dim1)
    assert np.array_equal(np.ascontiguousarray(img1).view(np.uint64),
                          np.ascontiguousarray(ref1).view(np.uint64))
    # the first result, held across the second call, was not reused for it
    assert img1 is not img
    assert np.array_equal(np.ascontiguousarray(img).view(np.uint64),
                          np.ascontiguousarray(ref).view(np.uint64))
    del img1
    img2 = FocalizzatoreBpPx(*args, precision="mixed")
    assert np.array_equal(np.ascontiguousarray(img2).view(np.uint64),
                          np.ascontiguousarray(ref).view(np.uint64))


def test_drop_in_from_memory_mapped_files(tmp_path):
    """Inputs memory-mapped from .dat files (as the reference's large-scene
    script maps them): the call takes the driver's staged copies for the
    file-backed raw rows, never in-place device reads of the mapping, and
    gives the in-memory call's image bit for bit."""
    sc = SCENES["small"]()
    args = _host_args(sc)
    ref = FocalizzatoreBpPx(*args, precision="mixed")
    raw = args[8]
    mm = np.memmap(tmp_path / "raw_f.dat", dtype=np.complex64, mode="w+", shape=raw.shape,
                   order="F")
    mm[...] = raw
    mm.flush()
    mapped = list(args)
    mapped[8] = np.memmap(tmp_path / "raw_f.dat", dtype=np.complex64, mode="r",
                          shape=raw.shape, order="F")
    img = FocalizzatoreBpPx(*mapped, precision="mixed")
    assert focuser.last_call["streamed"] and focuser.last_call["upload"] == "copy"
    assert np.array_equal(np.ascontiguousarray(img).view(np.uint64),
                          np.ascontiguousarray(ref).view(np.uint64))
