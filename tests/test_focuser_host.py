"""Host-side behaviour of the drop-in focusing call (no GPU needed)."""
import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import FocalizzatoreBpPx, FocalizzatoreBpCuPy_Batched, synth
from sar_backprojection_gb300.scene import flatten_f


def _args():
    return list(synth.focus_args(synth.generate(synth.config_small())))


def test_raw_data_must_be_2d():
    a = _args()
    a[8] = a[8].reshape(-1)
    with pytest.raises(ValueError, match="Raw_Data must be a 2D array"):
        FocalizzatoreBpPx(*a)


def test_dem_must_be_2d():
    a = _args()
    a[0] = a[0].reshape(-1)
    with pytest.raises(ValueError, match="xxg1 must be a 2D array"):
        FocalizzatoreBpPx(*a)


def test_size_mismatch_and_short_trajectory():
    a = _args()
    a[3] = a[3][:-1]
    with pytest.raises(ValueError, match="mask"):
        FocalizzatoreBpPx(*a)
    a = _args()
    a[5] = a[5][:100]
    with pytest.raises(ValueError, match="wgsx"):
        FocalizzatoreBpPx(*a)
    # the reference reads pulses 0 < a < Naz-1 only: Naz-1 points are enough,
    # Naz-2 are not
    naz = a[8].shape[1]
    a = _args()
    a[6] = a[6][:naz - 2]
    with pytest.raises(ValueError, match="wgsy"):
        FocalizzatoreBpPx(*a)
    a = _args()
    a[5], a[6], a[7] = a[5][:naz - 1], a[6][:naz - 1], a[7][:naz - 1]
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError, match="CUDA"):   # past the argument checks
            FocalizzatoreBpPx(*a)


def test_batched_rejects_bad_batch_size():
    with pytest.raises(ValueError):
        FocalizzatoreBpCuPy_Batched(*_args(), batch_size=0)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU error")
def test_no_cpu_fallback():
    with pytest.raises(RuntimeError, match="CUDA"):
        FocalizzatoreBpPx(*_args())


def test_flatten_matches_numpy_fortran_order():
    a = np.arange(24, dtype=np.int64).reshape(4, 6)
    for arr in (a, np.asfortranarray(a)):
        t = flatten_f(arr, np.int32, "cpu")
        assert t.dtype == torch.int32
        assert np.array_equal(t.numpy(), arr.astype(np.int32).flatten(order="F"))
    # reference dtype coercion: float index truncates, uint8 wraps
    f = np.array([[1.7, -2.2], [3.9, 4.0]])
    assert np.array_equal(flatten_f(f, np.int32, "cpu").numpy(),
                          f.astype(np.int32).flatten(order="F"))
    m = np.array([[257, 1], [2, -255]])
    assert np.array_equal(flatten_f(m, np.uint8, "cpu").numpy(),
                          m.astype(np.uint8).flatten(order="F"))


def test_drop_in_results_are_fresh_arrays():
    """The drop-in call returns a new array every call, as the reference's
    focusing call does (pages faulted in ahead by a helper thread): no
    result shares memory with another, whether or not the caller holds it."""
    import time
    from sar_backprojection_gb300.focuser import FreshImages
    pool = FreshImages(ahead=2)
    a = pool.get(4, 3)
    assert a.shape == (4, 3) and a.dtype == np.complex128 and a.flags.f_contiguous
    time.sleep(0.05)                                 # let the helper fill ahead
    b = pool.get(4, 3)
    assert b is not a and not np.shares_memory(a, b)
    a[...] = 1 + 2j
    del a
    c = pool.get(4, 3)
    assert not np.shares_memory(b, c) and (c == 0).all()
    assert pool.get(5, 3).shape == (5, 3)           # another shape
    held = [pool.get(2, 2) for _ in range(6)]
    assert all(not np.shares_memory(x, y) for i, x in enumerate(held) for y in held[i + 1:])


def test_scene_upload_mode_arguments_are_checked_before_the_device():
    from sar_backprojection_gb300.scene import scene_to_device
    a = _args()
    with pytest.raises(ValueError, match="raw_bins"):
        scene_to_device(*a, raw_bins="sometimes")
    with pytest.raises(ValueError, match="bound_host"):
        scene_to_device(*a, raw_bins="deferred")          # needs the pinned pair
    with pytest.raises(ValueError, match="h2d"):
        scene_to_device(*a, h2d="dma")


def test_read_bound_takes_the_deferred_pair_once():
    """read_bound turns the pair the device wrote into (bin_lo, bin_hi) and
    forgets the buffer, so a later call returns the same values."""
    from types import SimpleNamespace
    from sar_backprojection_gb300.scene import read_bound
    pair = torch.tensor([209, 1785], dtype=torch.int32)
    sc = SimpleNamespace(bound_host=pair, bin_lo=0, bin_hi=-1)
    assert read_bound(sc) == (209, 1785)
    assert sc.bound_host is None
    pair[:] = torch.tensor([1, 0], dtype=torch.int32)      # the slot's next job
    assert read_bound(sc) == (209, 1785)
    empty = SimpleNamespace(bound_host=torch.tensor([1, 0], dtype=torch.int32), bin_lo=0,
                            bin_hi=-1)
    lo, hi = read_bound(empty)
    assert lo > hi                                           # nothing reached



def test_serving_engine_checks_its_options_before_the_device():
    from sar_backprojection_gb300 import serve
    with pytest.raises(ValueError, match="h2d"):
        serve.ServingEngine(device="cpu", h2d="dma")
    with pytest.raises(ValueError, match="policy"):
        serve.ServingEngine(device="cpu", policy="lifo")


@pytest.mark.parametrize("naz,blocks,tail,head", [(40001, 8, 1, 0), (40001, 8, 3, 2),
                                                  (2001, 4, 0, 0), (37, 8, 2, 3),
                                                  (40001, 30, 4, 2)])
def test_stream_marks_cover_the_pulses_with_a_short_tail(naz, blocks, tail, head):
    from sar_backprojection_gb300.focuser import _stream_marks

    m = _stream_marks(naz, blocks, tail, head)
    assert m[-1] == naz and len(m) <= 32
    assert all(a <= b for a, b in zip(m, m[1:]))
    if head and len(m) == blocks + tail + head:
        assert m[0] == naz // (blocks << head)
    if len(m) == blocks + tail + head:
        # the final blocks halve
        lens = np.diff([0] + m)
        assert all(lens[-1 - h] <= (naz // blocks) // (1 << h) + 1 for h in range(tail))


def test_one_call_upload_takes_only_arrays_that_need_no_conversion():
    """The drop-in's one-call upload accepts column-major arrays of the
    reference's dtypes (NumPy F-order, a transposed C-contiguous tensor) and
    leaves everything else to the per-array path."""
    from sar_backprojection_gb300.focuser import _column_major_words

    f = np.asfortranarray(np.zeros((6, 4)))
    assert _column_major_words(f, torch.float64, 24, True) == f.__array_interface__["data"][0]
    assert _column_major_words(np.zeros((6, 4)), torch.float64, 24, True) is None   # C order
    assert _column_major_words(f.astype(np.float32), torch.float64, 24, True) is None
    assert _column_major_words(f, torch.float64, 23, True) is None                  # size
    assert _column_major_words(f[:, :3], torch.float64, 18, True) is not None        # F slice
    assert _column_major_words(f[::2], torch.float64, 12, True) is None              # strided
    t = torch.zeros((4, 6), dtype=torch.int32).t()
    assert _column_major_words(t, torch.int32, 24, True) == t.data_ptr()
    assert _column_major_words(t.t(), torch.int32, 24, True) is None
    w = np.zeros(11)
    assert _column_major_words(w, torch.float64, 10, False) is not None               # >= naz
    assert _column_major_words(w, torch.float64, 12, False) is None
    assert _column_major_words([1.0, 2.0], torch.float64, 2, False) is None


def test_file_mappings_are_recognised(tmp_path):
    """Memory-mapped inputs (and views of them) are kept off the in-place
    pageable path; ordinary arrays are not."""
    from sar_backprojection_gb300.focuser import _column_major_words, _file_backed

    p = tmp_path / "a.dat"
    np.zeros(24).tofile(p)
    mm = np.memmap(p, dtype=np.float64, mode="r", shape=(6, 4), order="F")
    assert _file_backed(mm) and _file_backed(mm.T) and _file_backed(mm[:, :2])
    assert _file_backed(np.asarray(mm))
    assert _column_major_words(mm, torch.float64, 24, True) is None
    assert not _file_backed(np.zeros((6, 4))) and not _file_backed(None)
    assert not _file_backed(np.array(mm, order="F"))         # a copy in ordinary memory
