"""Large-scene driver host logic: cursor and per-batch pulse ranges."""
import numpy as np

from sar_backprojection_gb300 import synth
from sar_backprojection_gb300.large_scene import Cursor, batch_pulse_range


def test_cursor_round_trip_and_match(tmp_path):
    p = tmp_path / "c.json"
    c = Cursor(10, 20, 30, 40, 5, next_batch=3)
    c.save(p)
    back = Cursor.load(p)
    assert back == c and back.matches(Cursor(10, 20, 30, 40, 5))
    assert not back.matches(Cursor(10, 20, 30, 41, 5))
    (tmp_path / "bad.json").write_text("{not json")
    assert Cursor.load(tmp_path / "bad.json") is None
    assert Cursor.load(tmp_path / "missing.json") is None


def test_batch_pulse_range_matches_brute_force():
    rng = np.random.default_rng(0)
    naz = 500
    idx = rng.integers(-20, naz + 20, (6, 7)).astype(np.int32)
    s = rng.choice([-9999, -3, -1, 0, 1, 7, 40, 41, 600], (6, 7)).astype(np.int32)
    m = rng.choice([0, 1, 2], (6, 7)).astype(np.uint8)
    lo, hi = batch_pulse_range(idx, s, m, naz)
    kept = []
    for i, sv, mv in zip(idx.ravel(), s.ravel(), m.ravel()):
        if mv != 1 or sv == -9999:
            continue
        jj = int(np.ceil(sv / 2.0)) * 2 + 1
        off = int(np.ceil(abs(sv) / 2.0))
        kept += [a for a in range(i - off, i - off + jj) if 0 < a < naz - 1]
    if kept:
        assert (lo, hi) == (min(kept), max(kept))
    else:
        assert (lo, hi) == (0, -1)


def test_azimuth_columns_transposes_grid_only():
    sc = synth.generate(synth.SceneSpec(name="t", seed=1, dim0=16, dim1=8, x0=495.0, naz=301,
                                        nra=96, near_range=3610.0, sint_lo=40, sint_hi=60))
    t = synth.azimuth_columns(sc)
    assert t["xxg1"].shape == (8, 16) and t["xxg1"].flags.f_contiguous
    assert np.array_equal(t["Index"], sc["Index"].T)
    assert t["RawData"] is sc["RawData"]


def test_file_io_reads_and_writes_byte_ranges(tmp_path):
    """Positional reads/writes split over threads land at the right offsets."""
    from sar_backprojection_gb300.large_scene import FileIO
    data = np.random.default_rng(1).integers(0, 255, 50_000_000, dtype=np.uint8)
    p = tmp_path / "f.bin"
    data.tofile(p)
    fio = FileIO(threads=4)
    fio.CHUNK = 1 << 20
    buf = np.empty(20_000_001, dtype=np.uint8)
    fio.read(p, buf, 12_345_678)
    assert np.array_equal(buf, data[12_345_678:32_345_679])
    out = tmp_path / "o.bin"
    np.zeros(30_000_000, dtype=np.uint8).tofile(out)
    fio.write(out, buf, 3)
    back = np.fromfile(out, dtype=np.uint8)
    assert np.array_equal(back[3:20_000_004], buf) and back[:3].sum() == 0
    fio.close()
