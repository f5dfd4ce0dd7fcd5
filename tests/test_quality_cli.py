"""The parity-report CLI reads every image format the reference writes or reads.

The reference's focusing script writes ``SlcPx_*_SplitF32.dat`` (all real
parts, then all imaginary parts, float32, column-major) and
``SlcPx_*_InterleavedF32.dat`` (float32 pairs) beside a complex128 ``.npy``
(sar_focuser_puntual_noui.py:440-469); its phase tool reads ``interleaved``,
``split`` and ``truth`` (complex64) layouts (compare_phase.py:8-37); the
README names ``SlcMatr_real.dat`` / ``SlcMatr_imag.dat`` (float64).  Files are
built here byte by byte the way those writers lay them out, and also through
``datfiles.write_slc``; every format must load to the same image, and the CLI
must report the same statistics as ``quality.compare`` on the arrays.
"""
import json

import numpy as np
import pytest

from sar_backprojection_gb300 import datfiles, quality

SHAPE = (40, 24)


def _image(seed):
    rng = np.random.default_rng(seed)
    img = rng.standard_normal(SHAPE) + 1j * rng.standard_normal(SHAPE)
    return np.asfortranarray(img)


def _reference_layouts(img, d):
    """The reference writers' byte layouts, restated with NumPy."""
    re = img.real.astype(np.float32).reshape(-1, order="F")
    im = img.imag.astype(np.float32).reshape(-1, order="F")
    split = d / "SlcPx_Python_Corrected_SplitF32.dat"
    with open(split, "wb") as f:
        re.tofile(f)
        im.tofile(f)
    inter = d / "SlcPx_Python_Corrected_InterleavedF32.dat"
    pairs = np.empty(2 * re.size, dtype=np.float32)
    pairs[0::2] = re
    pairs[1::2] = im
    pairs.tofile(inter)
    truth = d / "truth.dat"
    img.astype(np.complex64).reshape(-1, order="F").tofile(truth)
    npy = d / "SlcPx_Python_Corrected.npy"
    np.save(npy, img)
    return {"split": split, "interleaved": inter, "truth": truth, "npy": npy}


def test_every_reference_format_loads_the_same_image(tmp_path):
    img = _image(1)
    f32 = img.astype(np.complex64).astype(np.complex128)
    paths = _reference_layouts(img, tmp_path)
    for fmt in ("split", "interleaved", "truth"):
        got = quality.load_image(str(paths[fmt]), SHAPE, fmt)
        assert np.array_equal(got, f32), fmt
    assert np.array_equal(quality.load_image(str(paths["npy"]), SHAPE, "auto"), img)
    # auto by size: complex64 files read as interleaved (== truth)
    assert np.array_equal(quality.load_image(str(paths["interleaved"]), SHAPE), f32)
    written = datfiles.write_slc(tmp_path / "ours", img)
    assert (open(written["split_f32"], "rb").read() == open(paths["split"], "rb").read())
    assert (open(written["interleaved_f32"], "rb").read()
            == open(paths["interleaved"], "rb").read())
    assert np.array_equal(quality.load_image(written["complex"], SHAPE), img)
    assert np.array_equal(quality.load_image(written["complex"], SHAPE, "complex128"), img)
    for p in (written["real"], written["imag"], str(tmp_path / "ours")):
        assert np.array_equal(quality.load_image(p, SHAPE, "slcmatr"), img)


def test_cli_reports_the_statistics_of_compare(tmp_path, capsys):
    ref = _image(2)
    noisy = ref * np.exp(1j * 2e-3) + 1e-4 * _image(3)
    rpaths = _reference_layouts(ref, tmp_path)
    (tmp_path / "n").mkdir()
    npaths = _reference_layouts(noisy, tmp_path / "n")
    out = tmp_path / "cmp"
    stats = quality.main(["--file1", str(npaths["split"]), "--file2", str(rpaths["truth"]),
                          "--shape", f"{SHAPE[0]},{SHAPE[1]}", "--fmt1", "split",
                          "--fmt2", "truth", "--out", str(out)])
    printed = json.loads(capsys.readouterr().out)
    on_disk = json.loads((tmp_path / "cmp_statistics.json").read_text())
    want = quality.compare(noisy.astype(np.complex64), ref.astype(np.complex64))
    for s in (stats, printed, on_disk):
        assert s["coherence"] == pytest.approx(want["coherence"], rel=1e-12)
        assert s["rms_phase_mrad"] == pytest.approx(want["rms_phase_mrad"], rel=1e-12)
        assert s["phase"]["large_errors"] == want["phase"]["large_errors"]
    # positional spelling with space-separated shape, complex128 files
    w1 = datfiles.write_slc(tmp_path / "a", noisy)
    w2 = datfiles.write_slc(tmp_path / "b", ref)
    st2 = quality.main([w1["complex"], w2["complex"], "--shape", str(SHAPE[0]), str(SHAPE[1])])
    assert st2["rms_phase_mrad"] == pytest.approx(quality.compare(noisy, ref)["rms_phase_mrad"])
    # --no-mask keeps every pixel
    st3 = quality.main([w1["npy"], w2["npy"], "--shape", "40,24", "--no-mask"])
    assert st3["phase"]["valid_pixels"] == SHAPE[0] * SHAPE[1]


def test_cli_rejects_sizes_that_do_not_match(tmp_path):
    p = tmp_path / "odd.dat"
    np.zeros(7, dtype=np.float32).tofile(p)
    with pytest.raises(ValueError):
        quality.load_image(str(p), SHAPE)
    with pytest.raises(ValueError):
        quality.load_image(str(p), SHAPE, "split")
