"""GPU parity: the CUDA kernels (through the C ABI) against the oracle.

Bars:
* range-bin selection is bit-exact: per-pixel contributor counts and the
  per-pixel checksum of contributing (pulse, bin) pairs equal the oracle's;
* FP64 kernel values: |gpu - oracle| <= 1e-12*|oracle| + 1e-13*rms(oracle)
  per pixel (CUDA's vs the C library's double cos/sin are the only
  difference);
* mixed-precision kernel: coherence >= 0.9999 and RMS phase error <= 1 mrad
  against the FP64 oracle, relative L2 error <= 1e-3.
"""
import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden_scene
from oracle import oracle
from sar_backprojection_gb300 import _lib, focus, quality, scene_to_device, synth

pytestmark = pytest.mark.gpu

FP64_REL = 1e-12
FP64_ABS_RMS = 1e-13
MIXED_COHERENCE = 0.9999
MIXED_RMS_MRAD = 1.0
MIXED_REL_L2 = 1e-3

TUNINGS = ([dict(chunk=c, tile0=t0, tile1=t1, staged=0) for c in (32, 64)
            for (t0, t1) in ((32, 8), (64, 4), (16, 16))]
           + [dict(chunk=c, tile0=t0, tile1=t1, staged=s, window=w)
              for (c, s) in ((32, 1), (32, 2), (64, 1), (64, 2), (128, 1))
              for (t0, t1, w) in ((32, 8, 128), (64, 4, 128), (16, 16, 128), (16, 16, 160),
                                  (16, 16, 208), (16, 8, 128))]
           + [dict(chunk=c, tile0=t0, tile1=t1, staged=1, window=w, stage=16)
              for c in (32, 128) for (t0, t1, w) in ((16, 16, 160), (16, 8, 128))])
TUNING_IDS = [f"c{t['chunk']}_{t['tile0']}x{t['tile1']}_"
              + ({0: "l1", 1: "tma", 2: "queue"}[t['staged']])
              + (str(t['window']) if t['staged'] else "")
              + (f"s{t['stage']}" if 'stage' in t else "") for t in TUNINGS]


def run(scene, precision, tuning=None):
    ds = scene_to_device(*synth.focus_args(scene))
    res = focus(ds, precision, tuning=tuning, diagnostics=True)
    torch.cuda.synchronize()
    shape = (ds.dim0, ds.dim1)
    img = res.to_numpy(*shape)
    nv = res.nvalid.cpu().numpy().reshape(shape, order="F")
    cs = res.checksum.cpu().numpy().view(np.uint64).reshape(shape, order="F")
    ctr = res.counters.cpu().numpy() if res.counters is not None else None
    return img, nv, cs, ctr


def assert_fp64_close(img, ref):
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    err = np.abs(img - ref)
    bound = FP64_REL * np.abs(ref) + FP64_ABS_RMS * rms
    worst = np.argmax(err - bound)
    assert (err <= bound).all(), f"pixel {worst}: err {err.flat[worst]} > {bound.flat[worst]}"


def assert_mixed_quality(img, ref):
    q = quality.compare(img, ref)
    assert q["coherence"] >= MIXED_COHERENCE, q
    assert q["rms_phase_mrad"] <= MIXED_RMS_MRAD, q
    assert q["rel_l2"] <= MIXED_REL_L2, q
    return q


@pytest.fixture(scope="module")
def small():
    g = np.load(GOLDEN / "golden_small.npz")
    scene = synth.generate(synth.config_small(int(g["seed"])))
    return scene, g["image"]


@pytest.mark.parametrize("name", ["edges", "ties"])
def test_fp64_kernel_golden(name):
    scene, ref = load_golden_scene(name)
    img, nv, cs, _ = run(scene, "fp64")
    _, onv, ocs = oracle.focus_scene(scene)
    assert np.array_equal(nv, onv)
    assert np.array_equal(cs, ocs)
    assert_fp64_close(img, ref)


def test_fp64_kernel_small_workload(small):
    scene, ref = small
    img, nv, cs, _ = run(scene, "fp64")
    _, onv, ocs = oracle.focus_scene(scene)
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    assert_fp64_close(img, ref)


@pytest.mark.parametrize("name", ["edges", "ties"])
def test_mixed_kernel_golden(name):
    scene, ref = load_golden_scene(name)
    img, nv, cs, ctr = run(scene, "mixed")
    _, onv, ocs = oracle.focus_scene(scene)
    assert np.array_equal(nv, onv)
    assert np.array_equal(cs, ocs)
    assert_mixed_quality(img, ref)
    assert (img[onv == 0] == 0).all()


@pytest.mark.parametrize("tuning", TUNINGS, ids=TUNING_IDS)
def test_mixed_kernel_small_workload_tunings(small, tuning):
    scene, ref = small
    img, nv, cs, ctr = run(scene, "mixed", tuning)
    _, onv, ocs = oracle.focus_scene(scene)
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    assert_mixed_quality(img, ref)


def test_fast_path_equals_diagnostic_path(small):
    """The production launch (no checksum) gives the same image bits."""
    scene, _ = small
    ds = scene_to_device(*synth.focus_args(scene))
    a = focus(ds, "mixed").image.clone()
    b = focus(ds, "mixed", diagnostics=True).image
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    c = focus(ds, "fp64").image.clone()
    d = focus(ds, "fp64", diagnostics=True).image
    torch.cuda.synchronize()
    assert torch.equal(c, d)


@pytest.fixture(scope="module")
def full_scene():
    spec = synth.config_full()
    scene = synth.generate(spec, raw_device="cuda")
    return scene


@pytest.fixture(scope="module")
def full_oracle(full_scene):
    host = dict(full_scene)
    host["RawData"] = full_scene["RawData"].cpu()     # (nra, naz) view, pulse-major
    return oracle.focus_scene(host)


def test_full_workload_fp64(full_scene, full_oracle):
    """4000 x 250 pixels, 40001 pulses: FP64 kernel against the full oracle."""
    oimg, onv, ocs = full_oracle
    img, nv, cs, _ = run(full_scene, "fp64")
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    assert_fp64_close(img, oimg)


@pytest.mark.parametrize("tuning", [dict(chunk=64, tile0=32, tile1=8, staged=0),
                                    dict(chunk=32, tile0=16, tile1=16, staged=1, window=128),
                                    dict(chunk=32, tile0=16, tile1=16, staged=1, window=160),
                                    dict(chunk=32, tile0=16, tile1=8, staged=1, window=128),
                                    dict(chunk=32, tile0=64, tile1=4, staged=1, window=128),
                                    dict(chunk=32, tile0=16, tile1=16, staged=2, window=160),
                                    dict(chunk=32, tile0=16, tile1=8, staged=2, window=128),
                                    dict(chunk=64, tile0=16, tile1=16, staged=1, window=160),
                                    dict(chunk=64, tile0=16, tile1=16, staged=1, window=128),
                                    dict(chunk=64, tile0=32, tile1=8, staged=2, window=128),
                                    dict(chunk=128, tile0=16, tile1=16, staged=1, window=160),
                                    dict(chunk=128, tile0=16, tile1=16, staged=1, window=208),
                                    dict(chunk=128, tile0=16, tile1=16, staged=1, window=192),
                                    dict(chunk=128, tile0=16, tile1=16, staged=3, window=208),
                                    dict(chunk=128, tile0=16, tile1=16, staged=1, window=160,
                                         stage=16),
                                    dict(chunk=64, tile0=16, tile1=8, staged=2, window=128,
                                         stage=16)],
                         ids=["c64_l1", "tma_16x16w128", "tma_16x16w160", "tma_16x8w128",
                              "tma_64x4w128", "queue_16x16w160", "queue_16x8w128",
                              "c64_tma_16x16w160", "c64_tma_16x16w128", "c64_queue_32x8w128",
                              "c128_tma_16x16w160", "c128_tma_16x16w208", "c128_tma_16x16w192",
                              "c128_byend_16x16w208", "c128_tma_16x16w160s16",
                              "c64_queue_16x8w128s16"])
def test_full_workload_mixed(full_scene, full_oracle, tuning):
    """Mixed kernel variants against the full oracle image."""
    oimg, onv, ocs = full_oracle
    mimg, mnv, mcs, ctr = run(full_scene, "mixed", tuning)
    assert np.array_equal(mnv, onv) and np.array_equal(mcs, ocs)
    q = assert_mixed_quality(mimg, oimg)
    assert ctr[3] == 0                                 # no bounded wait gave up
    print("full workload mixed", tuning, {k: q[k] for k in ("rel_l2", "coherence",
                                                             "rms_phase_mrad")},
          "counters:", ctr[:4])


@pytest.mark.parametrize("tiling", [(16, 16, 160), (32, 8, 128)], ids=["16x16w160", "32x8w128"])
def test_tile_queue_matches_one_cta_per_tile(full_scene, tiling):
    """The persistent queue grid runs the same per-tile code: bit-identical."""
    t0, t1, w = tiling
    a = run(full_scene, "mixed", dict(chunk=32, tile0=t0, tile1=t1, staged=1, window=w))
    b = run(full_scene, "mixed", dict(chunk=32, tile0=t0, tile1=t1, staged=2, window=w))
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[3][:3], b[3][:3]) and b[3][3] == 0


def image_of(image: torch.Tensor, shape) -> np.ndarray:
    """complex128 (dim0, dim1) host image of a device (npix, 2) float64 image."""
    flat = image.cpu().numpy().view(np.complex128).reshape(-1)
    return np.reshape(flat, shape, order="F")


def _bench_tunings():
    """The staged candidates bench.py times on the full workload (it measures
    the first within 1 % of the fastest)."""
    import bench
    return [dict(zip(bench.TUNING_FIELDS, c)) for c in bench.AUTOTUNE_CANDIDATES]


@pytest.mark.parametrize("tuning", _bench_tunings(),
                         ids=lambda t: f"c{t['chunk']}_{t['tile0']}x{t['tile1']}w{t['window']}")
def test_full_workload_production_launch(full_scene, full_oracle, tuning):
    """The launch bench.py times: no checksum output (the production kernel
    instantiation), each of the bench's candidate tunings, on the full
    workload.  Its image must equal the diagnostic launch's bit for bit, the
    diagnostic launch's range bins must equal the oracle's, and the image must
    meet the mixed-precision bars against the oracle's image."""
    oimg, onv, ocs = full_oracle
    ds = scene_to_device(*synth.focus_args(full_scene))
    prod = focus(ds, "mixed", tuning=tuning).check()
    prod_img = prod.image.clone()
    diag = focus(ds, "mixed", tuning=tuning, diagnostics=True).check()
    torch.cuda.synchronize()
    assert torch.equal(prod_img, diag.image)
    shape = (ds.dim0, ds.dim1)
    nv = diag.nvalid.cpu().numpy().reshape(shape, order="F")
    cs = diag.checksum.cpu().numpy().view(np.uint64).reshape(shape, order="F")
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    assert int(diag.counters[3].item()) == 0
    img = image_of(prod_img, shape)
    q = assert_mixed_quality(img, oimg)
    print("production launch", tuning, {k: q[k] for k in ("rel_l2", "coherence",
                                                          "rms_phase_mrad")})


@pytest.mark.parametrize("upload,pinned", [("signal", True), ("sm", True), ("copy", True),
                                           ("signal", False)])
def test_full_workload_streamed_drop_in(full_scene, full_oracle, upload, pinned, monkeypatch):
    """The drop-in call as the bench's e2e measures it: host inputs in the
    reference's layout, precision="mixed" with the bench's preferred tuning,
    the reachable range bins streamed up in pulse blocks while focusing runs
    (by each upload mode: SM loads per block, one persistent block copy that
    signals each block through a device flag, the copy engine; page-locked
    raw rows, and pageable ones, which the SM-load modes read in place on a
    device that reaches pageable memory and the copy engine takes elsewhere).
    The returned image must equal the resident launch of the same tuning bit
    for bit (whose range bins equal the oracle's) and meet the bars against
    the oracle."""
    from sar_backprojection_gb300 import FocalizzatoreBpPx, focuser

    monkeypatch.setattr(focuser, "STREAM_UPLOAD", upload)
    oimg, onv, ocs = full_oracle
    tuning = _bench_tunings()[0]
    host = dict(full_scene)
    raw = full_scene["RawData"]                          # (nra, naz), pulse-major memory
    if pinned:
        rows = torch.empty((raw.shape[1], raw.shape[0]), dtype=raw.dtype, pin_memory=True)
        rows.copy_(raw.t())
        host["RawData"] = rows.t()
    else:
        host["RawData"] = raw.cpu()
    for _ in range(2):                                   # second call: next flag generation
        img = FocalizzatoreBpPx(*synth.focus_args(host), precision="mixed", tuning=tuning)
    assert focuser.last_call["streamed"]
    # pageable rows take the copy engine unless the device reads pageable
    # host memory in place
    reachable = pinned or bool(_lib.load().sarbp_device_reads_pageable())
    assert focuser.last_call["upload"] == (upload if reachable else "copy")
    if upload == "signal" and reachable:
        assert focuser.last_call["small_upload"] == "one-call"
    assert img.shape == (4000, 250) and img.dtype == np.complex128
    ds = scene_to_device(*synth.focus_args(full_scene))
    diag = focus(ds, "mixed", tuning=tuning, diagnostics=True).check()
    torch.cuda.synchronize()
    shape = (ds.dim0, ds.dim1)
    assert np.array_equal(img, image_of(diag.image, shape))
    nv = diag.nvalid.cpu().numpy().reshape(shape, order="F")
    cs = diag.checksum.cpu().numpy().view(np.uint64).reshape(shape, order="F")
    assert np.array_equal(nv, onv) and np.array_equal(cs, ocs)
    assert_mixed_quality(img, oimg)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_trajectory_of_naz_minus_one_points(precision):
    """The reference reads the trajectory only at pulses 0 < a < Naz-1, so it
    accepts Naz-1 points (sar_focuser_puntual_noui.py:46-55): on the edge-case
    scene (apertures at pulses 0, 1, Naz-2, Naz-1) a trajectory one point
    short gives the oracle's range bins and the same image bits as the full
    one."""
    scene, ref = load_golden_scene("edges")
    naz = scene["RawData"].shape[1]
    short = dict(scene)
    for k in ("wgsx", "wgsy", "wgsz"):
        short[k] = np.ascontiguousarray(scene[k][: naz - 1])
    full = run(scene, precision)
    cut = run(short, precision)
    for x, y in zip(full[:3], cut[:3]):
        assert np.array_equal(x, y)
    _, onv, ocs = oracle.focus_scene(short)
    assert np.array_equal(cut[1], onv) and np.array_equal(cut[2], ocs)
