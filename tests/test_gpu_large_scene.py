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
