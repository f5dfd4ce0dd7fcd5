"""The oracle against golden vectors produced by the reference itself.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs the
unmodified reference FocalizzatoreBpPx (sar_focuser_puntual_noui.py:149).
The oracle must reproduce them bit for bit.
"""
import numpy as np
import pytest

from conftest import GOLDEN, load_golden_scene
from oracle import oracle
from sar_backprojection_gb300 import synth


def bits(a):
    """Raw IEEE bit patterns of a complex128 array (any memory order)."""
    return np.ascontiguousarray(a).reshape(-1).view(np.uint64)


@pytest.mark.parametrize("name", ["edges", "ties"])
def test_oracle_matches_reference_bitwise(name):
    scene, ref = load_golden_scene(name)
    img, nv, cs = oracle.focus_scene(scene)
    assert img.shape == ref.shape and img.dtype == np.complex128
    assert np.array_equal(bits(img), bits(ref))


def test_oracle_matches_reference_small_workload():
    g = np.load(GOLDEN / "golden_small.npz")
    scene = synth.generate(synth.config_small(int(g["seed"])))
    assert synth.input_digest(scene) == str(g["digest"]), \
        "regenerated small-workload inputs differ from the ones the fixture was made from"
    img, nv, cs = oracle.focus_scene(scene)
    assert np.array_equal(bits(img), bits(g["image"]))
    # every pixel of the small workload sees its whole 401-pulse aperture
    assert (nv == 401).all()


def test_oracle_edge_counts():
    scene, _ = load_golden_scene("edges")
    _, nv, _ = oracle.focus_scene(scene)
    # Sint -9999, -3, -2 -> nothing; -1 and 0 -> one pulse; 1, 2 -> three;
    # 3 -> five; 5000 -> every kept pulse 0 < a < Naz-1.
    naz = scene["wgsx"].size
    assert list(nv[0:9, 0]) == [0, 0, 0, 1, 1, 3, 3, 5, naz - 2]
    # mask 0, 2 and 255 are all "not 1"
    assert list(nv[9:12, 0]) == [0, 0, 0]
    # pixels whose range bins cross 0 keep only part of the aperture
    assert (nv[19:22, 0] > 0).all() and (nv[19:22, 0] < 41).all()


def test_oracle_ties_round_half_even():
    scene, _ = load_golden_scene("ties")
    # pixel (0, 0) sits at the origin: every even pulse is an exact tie
    # (R - near)/dra = n + 0.5; count and checksum must follow half-to-even.
    _, nv, cs = oracle.focus_scene(scene)
    near, dra = float(scene["NearRange"]), float(scene["DeltaRange"])
    nra = scene["RawData"].shape[0]
    naz = scene["wgsx"].size
    s, idx = int(scene["Sint"][0, 0]), int(scene["Index"][0, 0])
    half = (s + 1) // 2
    expect_n, expect_cs = 0, 0
    for a in range(idx - half, idx - half + 2 * half + 1):
        if not 0 < a < naz - 1:
            continue
        d = np.array([0.0 - scene["wgsx"][a], 0.0 - scene["wgsy"][a], 0.0 - scene["wgsz"][a]])
        r = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        b = int(np.round((r - near) / dra))
        if 0 <= b < nra - 1:
            expect_n += 1
            expect_cs = (expect_cs + oracle.mix64(a, b)) % (1 << 64)
    assert nv[0, 0] == expect_n
    assert int(cs[0, 0]) == expect_cs


def test_oracle_thread_count_invariant():
    scene, _ = load_golden_scene("edges")
    a = oracle.focus_scene(scene, nthreads=1)
    b = oracle.focus_scene(scene, nthreads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_oracle_pixel_subset_matches_full():
    scene, _ = load_golden_scene("edges")
    full, nv, cs = oracle.focus_scene(scene)
    pix = np.array([0, 5, 17, 40, 77, 150, 191])
    v, n2, c2 = oracle.focus_scene(scene, pixels=pix)
    assert np.array_equal(v, full.reshape(-1, order="F")[pix])
    assert np.array_equal(n2, nv.reshape(-1, order="F")[pix])
    assert np.array_equal(c2, cs.reshape(-1, order="F")[pix])
