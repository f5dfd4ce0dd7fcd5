"""Large-scene driver: azimuth batches + resume equal the single-call image."""
import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import FocalizzatoreBpPx, datfiles, synth
from sar_backprojection_gb300.large_scene import Cursor, LargeSceneFocuser

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    spec = synth.scaled_full(77, 600, 64, 6001, 800, 1200)
    sc = synth.azimuth_columns(synth.generate(spec, raw_device="cuda"))
    sc["RawData"] = sc["RawData"].cpu().numpy()            # (nra, naz), column-major bytes
    d = tmp_path_factory.mktemp("large")
    datfiles.save_scene(d, sc)
    dim0, dim1 = sc["xxg1"].shape
    nra, naz = sc["RawData"].shape
    return d, sc, (dim0, dim1, nra, naz)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_batches_equal_single_call(files, tmp_path):
    d, sc, (dim0, dim1, nra, naz) = files
    ref = FocalizzatoreBpPx(*synth.focus_args(sc), precision="mixed")
    lf = LargeSceneFocuser(tmp_path / "slc.dat", batch_cols=96, block_pulses=1024)
    out = lf.focus_files(d, dim0, dim1, nra, naz)
    assert np.array_equal(_bits(np.asarray(out)), _bits(ref))
    assert Cursor.load(tmp_path / "slc.dat.cursor").next_batch == (dim1 + 95) // 96
    # in-memory arguments (no files: arrays read where they lie)
    lf2 = LargeSceneFocuser(tmp_path / "slc2.dat", batch_cols=96, block_pulses=1024)
    out2 = lf2.focus(*synth.focus_args(sc))
    assert np.array_equal(_bits(np.asarray(out2)), _bits(ref))


def test_resume_after_interruption(files, tmp_path):
    d, sc, (dim0, dim1, nra, naz) = files
    ref = FocalizzatoreBpPx(*synth.focus_args(sc), precision="mixed")
    lf = LargeSceneFocuser(tmp_path / "slc.dat", batch_cols=128, block_pulses=2048)
    lf.focus_files(d, dim0, dim1, nra, naz, max_batches=2)
    assert Cursor.load(tmp_path / "slc.dat.cursor").next_batch == 2
    lf2 = LargeSceneFocuser(tmp_path / "slc.dat", batch_cols=128, block_pulses=2048)
    out = lf2.focus_files(d, dim0, dim1, nra, naz)
    assert np.array_equal(_bits(np.asarray(out)), _bits(ref))
    torch.cuda.synchronize()


def test_above_l2_scene_against_the_oracle(tmp_path_factory):
    """A scene whose raw data (610 MB) exceed L2: the driver's column batches,
    streamed upload and an interruption + resume, with the diagnostic outputs,
    against the oracle on every pixel: contributor counts and range-bin
    checksums bit-exact, the image within the mixed-precision bars."""
    from oracle import oracle
    from sar_backprojection_gb300 import quality

    spec = synth.scaled_full(78, 400, 96, 16001, 1200, 1800)
    sc = synth.azimuth_columns(synth.generate(spec, raw_device="cuda"))
    d = tmp_path_factory.mktemp("above_l2")
    datfiles.save_scene(d, sc)
    dim0, dim1 = sc["xxg1"].shape
    nra, naz = sc["RawData"].shape
    host = dict(sc)
    host["RawData"] = sc["RawData"].cpu()
    oimg, onv, ocs = oracle.focus_scene(host)
    out = d / "slc.dat"
    lf = LargeSceneFocuser(out, batch_cols=64, block_pulses=4096, diagnostics=True)
    lf.focus_files(d, dim0, dim1, nra, naz, max_batches=3)
    assert Cursor.load(str(out) + ".cursor").next_batch == 3
    lf2 = LargeSceneFocuser(out, batch_cols=64, block_pulses=4096, diagnostics=True)
    img = np.asarray(lf2.focus_files(d, dim0, dim1, nra, naz))
    torch.cuda.synchronize()
    assert np.array_equal(np.asarray(lf2.nvalid), onv)
    assert np.array_equal(np.asarray(lf2.checksum), ocs)
    q = quality.compare(img, oimg)
    assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0 and q["rel_l2"] <= 1e-3, q
