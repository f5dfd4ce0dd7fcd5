"""The reference's .dat formats: round trips, loaders and their error paths."""
import numpy as np
import pytest

from sar_backprojection_gb300 import datfiles, synth


@pytest.fixture
def tiny_scene():
    spec = synth.SceneSpec(name="tiny", seed=3, dim0=16, dim1=8, x0=495.0, naz=301, nra=96,
                           near_range=3610.0, sint_lo=40, sint_hi=60)
    return synth.generate(spec)


def test_scene_round_trip(tmp_path, tiny_scene):
    names = datfiles.save_scene(tmp_path, tiny_scene)
    assert names["xxg1"] == "Dem_x_Dbl16x8.dat"
    assert names["RawData"] == "RawData_Cmplx_96x301.dat"
    assert names["wgsx"] == "Traiett_x_Dbl301.dat"
    back = datfiles.load_scene(tmp_path, 16, 8, 96, 301)
    for k in ("xxg1", "yyg1", "zzg1", "Mask", "Index", "Sint", "wgsx", "wgsy", "wgsz",
              "RawData"):
        assert back[k].dtype == np.asarray(tiny_scene[k]).dtype, k
        assert np.array_equal(back[k], tiny_scene[k]), k
    for k in ("NearRange", "DeltaRange", "Lambda"):
        assert back[k] == tiny_scene[k]
    # column-major on disk: element (1, 0) follows (0, 0)
    raw = np.fromfile(tmp_path / names["Sint"], dtype=np.int32)
    assert raw[1] == tiny_scene["Sint"][1, 0]


def test_scene_round_trip_from_a_tensor(tmp_path, tiny_scene):
    """Raw data held as a (Nra, Naz) tensor view of pulse-major storage (the
    GPU generator's form) is written in pulse-row blocks: same file bytes."""
    import torch
    sc = dict(tiny_scene)
    rows = torch.from_numpy(np.ascontiguousarray(np.asarray(tiny_scene["RawData"]).T))
    sc["RawData"] = rows.t()
    names = datfiles.save_scene(tmp_path / "t", sc)
    datfiles.save_scene(tmp_path / "n", tiny_scene)
    a = (tmp_path / "t" / names["RawData"]).read_bytes()
    assert a == (tmp_path / "n" / names["RawData"]).read_bytes()


def test_raw_interleaved_layout(tmp_path):
    raw = (np.arange(12, dtype=np.float32) + 1j * -np.arange(12, dtype=np.float32))
    raw = np.asfortranarray(raw.reshape(3, 4, order="F").astype(np.complex64))
    p = tmp_path / "RawData_Cmplx_3x4.dat"
    datfiles.write_dat(p, raw)
    f = np.fromfile(p, dtype=np.float32)
    # (r, a) at byte 8*(a*Nra + r): interleaved re, im
    assert f[2 * (2 * 3 + 1)] == raw[1, 2].real and f[2 * (2 * 3 + 1) + 1] == raw[1, 2].imag
    assert np.array_equal(datfiles.load_raw_strict(p, 3, 4), raw)


def test_raw_split_format(tmp_path):
    raw = np.asfortranarray((np.arange(6) + 10j * np.arange(6)).reshape(2, 3).astype(np.complex64))
    p = tmp_path / "split.dat"
    with open(p, "wb") as fh:
        raw.real.reshape(-1, order="F").astype(np.float32).tofile(fh)
        raw.imag.reshape(-1, order="F").astype(np.float32).tofile(fh)
    assert np.array_equal(datfiles.load_raw_strict(p, 2, 3, fmt="split"), raw)


def test_strict_loader_rejects_size_mismatch(tmp_path):
    p = tmp_path / "bad.dat"
    np.zeros(2 * 5 * 7 + 2, dtype=np.float32).tofile(p)
    with pytest.raises(IOError, match="does not match"):
        datfiles.load_raw_strict(p, 5, 7)


def test_tolerant_loader_odd_and_reshaped(tmp_path):
    p = tmp_path / "odd.dat"
    data = np.arange(2 * 4 * 6 + 1, dtype=np.float32)        # one float too many
    data.tofile(p)
    raw, nra, naz = datfiles.load_raw_data(tmp_path, "odd.dat", 4, 99)
    assert (nra, naz) == (4, 6)
    assert raw[1, 0] == data[2] + 1j * data[3]
    # not divisible by Nra -> nearest factor pair below sqrt
    p2 = tmp_path / "f.dat"
    np.arange(2 * 35, dtype=np.float32).tofile(p2)          # 35 complex = 5 x 7
    raw, nra, naz = datfiles.load_raw_data(tmp_path, "f.dat", 4, 9)
    assert (nra, naz) == (5, 7)


def test_memmap_validator(tmp_path):
    p = tmp_path / "m.dat"
    np.zeros(6 * 10, dtype=np.complex64).tofile(p)
    assert datfiles.validate_raw_dims(p, 6, 10) == (6, 10)
    assert datfiles.validate_raw_dims(p, 6, 99) == (6, 10)       # Naz from Nra
    assert datfiles.validate_raw_dims(p, 7, 10) == (6, 10)       # Nra from Naz
    with pytest.raises(ValueError, match="reconcile"):
        datfiles.validate_raw_dims(p, 7, 11)
    q = tmp_path / "n.dat"
    np.zeros(13, dtype=np.float32).tofile(q)
    with pytest.raises(ValueError, match="multiple"):
        datfiles.validate_raw_dims(q, 1, 1)
    with pytest.raises(FileNotFoundError):
        datfiles.validate_raw_dims(tmp_path / "missing.dat", 1, 1)
    mm = datfiles.open_raw_memmap(p, 6, 10)
    assert mm.shape == (6, 10) and mm.dtype == np.complex64


def test_trajectory_reconciliation():
    raw = np.zeros((4, 10), dtype=np.complex64)
    t = np.arange(8.0)
    r, x, y, z = datfiles.reconcile_trajectory(raw, t, t, t)
    assert r.shape == (4, 8) and len(x) == 8
    t2 = np.arange(12.0)
    r, x, y, z = datfiles.reconcile_trajectory(raw, t2, t2, t2)
    assert r.shape == (4, 10) and len(x) == 10


def test_slc_writers_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = (rng.standard_normal((40, 25)) + 1j * rng.standard_normal((40, 25)))
    paths = datfiles.write_slc(tmp_path, img)
    shape = img.shape
    assert np.array_equal(datfiles.read_slc(paths["complex"], shape, "complex"), img)
    assert np.array_equal(datfiles.read_slc(paths["npy"], shape, "npy"), img)
    assert np.array_equal(datfiles.read_slc(paths["real"], shape, "real"), img.real)
    assert np.array_equal(datfiles.read_slc(paths["imag"], shape, "imag"), img.imag)
    s = datfiles.read_slc(paths["split_f32"], shape, "split_f32")
    assert np.allclose(s, img, rtol=1e-6, atol=1e-6)
    i = datfiles.read_slc(paths["interleaved_f32"], shape, "interleaved_f32")
    assert np.allclose(i, img, rtol=1e-6, atol=1e-6)
    # the visualiser reads SlcMatr_real as (D1, D0) C-order: same bytes
    vis = np.fromfile(paths["real"], dtype=np.float64).reshape(25, 40)
    assert np.array_equal(vis.T, img.real)
