"""Host-to-device copies by SM loads (sarbp_upload_raw_bins_sm,
sarbp_copy_to_device_sm) give the copy engine's bytes, reject memory the
device cannot load from, and the serving engine that uses them for pinned
job inputs still gives every job the image it gets alone."""
import ctypes as C

import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import _lib, batch, focus, scene_to_device, serve, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return _lib.load()


def _stream():
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("naz,nra,dpitch,lo,nb", [
    (257, 1001, 1002, 123, 517),     # odd source pitch: complex64 words
    (257, 1000, 1000, 123, 517),     # even pitches, odd start and end: head and tail bins
    (257, 1000, 1002, 122, 518),     # even start and end: pairs only
    (257, 1000, 1000, 123, 518),     # odd start, even end
    (64, 4762, 4762, 209, 1577),     # the full workload's reachable bins
    (3, 8, 8, 1, 1),                 # one bin, odd: head only
    (3, 8, 8, 2, 1),                 # one bin, even: tail only
])
def test_raw_bins_match_the_copy_engine(lib, naz, nra, dpitch, lo, nb):
    host = torch.randn((naz, nra, 2), dtype=torch.float32).pin_memory()
    a = torch.full((naz, dpitch, 2), 7.0, device="cuda")
    b = a.clone()
    _lib.check(lib.sarbp_upload_raw_bins(a.data_ptr(), dpitch, host.data_ptr(), nra, lo, nb,
                                         naz, _stream()))
    _lib.check(lib.sarbp_upload_raw_bins_sm(b.data_ptr(), dpitch, host.data_ptr(), nra, lo, nb,
                                            naz, _stream()))
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert torch.equal(b[:, lo:lo + nb].cpu(), host[:, lo:lo + nb])
    assert bool((b[:, :lo] == 7.0).all()) and bool((b[:, lo + nb:] == 7.0).all())


@pytest.mark.parametrize("offset,size", [(0, 0), (0, 1), (3, 5), (5, 4096), (16, 1 << 20),
                                         (7, (1 << 20) + 13), (0, 3_000_001)])
def test_bytes_match(lib, offset, size):
    src = torch.randint(0, 256, (size + 64,), dtype=torch.uint8).pin_memory()
    dst = torch.zeros(size + 64, dtype=torch.uint8, device="cuda")
    for dofs in (0, 1, offset % 16):
        dst.zero_()
        _lib.check(lib.sarbp_copy_to_device_sm(dst.data_ptr() + dofs, src.data_ptr() + offset,
                                               size, _stream()))
        torch.cuda.synchronize()
        got = dst.cpu()
        assert torch.equal(got[dofs:dofs + size], src[offset:offset + size])
        assert int(got[:dofs].sum()) == 0 and int(got[dofs + size:].sum()) == 0


@pytest.mark.parametrize("naz,nra,dpitch,lo,nb,ends,ctas", [
    (257, 1000, 1002, 123, 517, [40, 41, 41, 200, 257], 7),   # an empty block
    (64, 4762, 4762, 209, 1577, [8 * k for k in range(1, 9)], 32),
    (5, 8, 8, 1, 1, [5], 64),                                  # more CTAs than rows
])
def test_signalled_blocks_match_the_copy_engine(lib, naz, nra, dpitch, lo, nb, ends, ctas):
    """The persistent block copy writes the copy engine's bytes, and after it
    every block's flag holds the call's generation; a stream held behind the
    last flag sees every row."""
    host = torch.randn((naz, nra, 2), dtype=torch.float32).pin_memory()
    a = torch.full((naz, dpitch, 2), 7.0, device="cuda")
    b = a.clone()
    flags = torch.zeros(32, dtype=torch.int32, device="cuda")
    counters = torch.zeros(32, dtype=torch.int32, device="cuda")
    e = np.asarray(ends, dtype=np.int64)
    _lib.check(lib.sarbp_upload_raw_bins(a.data_ptr(), dpitch, host.data_ptr(), nra, lo, nb,
                                         naz, _stream()))
    for gen in (1, 2):
        copy = torch.cuda.Stream()
        copy.wait_stream(torch.cuda.current_stream())
        _lib.check(lib.sarbp_upload_raw_blocks_sm(
            b.data_ptr(), dpitch, host.data_ptr(), nra, lo, nb, e.ctypes.data, len(ends),
            flags.data_ptr(), counters.data_ptr(), gen, ctas, copy.cuda_stream))
        user = torch.cuda.Stream()
        _lib.check(lib.sarbp_stream_wait_flag(user.cuda_stream,
                                              flags.data_ptr() + 4 * (len(ends) - 1), gen))
        with torch.cuda.stream(user):
            seen = b.clone()
        torch.cuda.synchronize()
        assert torch.equal(seen, a)
        assert flags[:len(ends)].tolist() == [gen] * len(ends)
        assert counters[:len(ends)].tolist() == [ctas] * len(ends)


@pytest.mark.parametrize("where", ["pinned", "device"])
@pytest.mark.parametrize("bound", [(123, 639), (0, 5000), (-7, 3), (1, 0), (900, 100)])
def test_blocks_read_their_bound_from_memory(lib, where, bound):
    """The bound-reading block copy equals the copy engine over the bound
    clipped to the rows; an empty bound copies nothing and still sets every
    flag."""
    naz, nra = 97, 1000
    host = torch.randn((naz, nra, 2), dtype=torch.float32).pin_memory()
    b = torch.tensor(bound, dtype=torch.int32)
    b = b.pin_memory() if where == "pinned" else b.cuda()
    lo, hi = max(bound[0], 0), min(bound[1], nra - 1)
    a = torch.full((naz, nra, 2), 7.0, device="cuda")
    got = a.clone()
    if hi >= lo:
        _lib.check(lib.sarbp_upload_raw_bins(a.data_ptr(), nra, host.data_ptr(), nra, lo,
                                             hi - lo + 1, naz, _stream()))
    flags = torch.zeros(32, dtype=torch.int32, device="cuda")
    counters = torch.zeros(32, dtype=torch.int32, device="cuda")
    ends = np.asarray([10, 50, 97], dtype=np.int64)
    _lib.check(lib.sarbp_upload_raw_blocks_bound_sm(
        got.data_ptr(), nra, host.data_ptr(), nra, b.data_ptr(), ends.ctypes.data, 3,
        flags.data_ptr(), counters.data_ptr(), 5, 16, _stream()))
    torch.cuda.synchronize()
    assert torch.equal(got, a)
    assert flags[:3].tolist() == [5, 5, 5]


def test_pageable_memory_is_read_in_place_or_rejected(lib):
    """Plain (pageable) host memory: on a device that reaches it through the
    host's page tables every SM-load copy reads it in place and the SM-store
    download writes it, with the copy engine's bytes; elsewhere each call
    refuses it before any launch."""
    rng = np.random.default_rng(3)
    src = rng.integers(0, 256, 4096 + 64, dtype=np.uint8)
    off = (-src.ctypes.data) % 16
    src = src[off:off + 4096]                            # 16-byte aligned, not page-locked
    dst = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    ends = np.asarray([3, 8], dtype=np.int64)
    flags = torch.zeros(4, dtype=torch.int32, device="cuda")
    calls = [
        lambda d: lib.sarbp_copy_to_device_sm(d.data_ptr(), src.ctypes.data, 4096, _stream()),
        lambda d: lib.sarbp_upload_raw_bins_sm(d.data_ptr(), 64, src.ctypes.data, 64, 0, 64, 8,
                                               _stream()),
        lambda d: lib.sarbp_upload_raw_blocks_sm(d.data_ptr(), 64, src.ctypes.data, 64, 0, 64,
                                                 ends.ctypes.data, 2, flags.data_ptr(),
                                                 flags.data_ptr() + 8, 1, 4, _stream()),
    ]
    want = torch.from_numpy(src.copy())
    if lib.sarbp_device_reads_pageable():
        for call in calls:
            dst.zero_()
            _lib.check(call(dst))
            torch.cuda.synchronize()
            assert torch.equal(dst.cpu(), want)
        back = np.zeros(4096 + 7, dtype=np.uint8)
        _lib.check(lib.sarbp_copy_to_host_sm(back.ctypes.data + 7, dst.data_ptr(), 4096,
                                             _stream()))
        torch.cuda.synchronize()
        assert np.array_equal(back[7:], src) and not back[:7].any()
    else:
        for call in calls:
            assert call(dst) == _lib.SARBP_EINVAL and "page-locked" in _lib.last_error()
        back = np.zeros(4096, dtype=np.uint8)
        assert lib.sarbp_copy_to_host_sm(back.ctypes.data, dst.data_ptr(), 4096,
                                         _stream()) == _lib.SARBP_EINVAL


def _pinned_args(sc):
    args = list(synth.focus_args(sc))
    for i in (0, 1, 2, 3, 4, 5, 6, 7, 8, 12):
        a = np.asarray(args[i])
        t = torch.from_numpy(np.ascontiguousarray(a.T) if a.ndim == 2 else a)
        args[i] = t.pin_memory().t() if a.ndim == 2 else t.pin_memory()
    return tuple(args)


def test_serving_with_pinned_inputs_matches_alone(lib):
    sizes = [(128, 32, 2001, 200, 260), (96, 40, 2401, 900, 1300), (160, 64, 3001, 600, 800)]
    arrivals = serve.poisson_arrivals(6, rate_per_s=400.0, seed=5)
    jobs = []
    for i in range(6):
        d0, d1, naz, s_lo, s_hi = sizes[i % 3]
        sc = synth.generate(synth.scaled_full(300 + i, d0, d1, naz, s_lo, s_hi))
        jobs.append(serve.Job(job_id=i, args=_pinned_args(sc), arrival=float(arrivals[i])))
    tuning = batch.staged_tuning()
    rep = serve.ServingEngine(budget_bytes=8 * serve.GB, max_slots=4, wave_items=64,
                              tuning=tuning).run(jobs)
    assert rep.summary()["completed"] == len(jobs)
    for j in jobs:
        ds = scene_to_device(*j.args, device="cuda")
        alone = focus(ds, "mixed", tuning=tuning)
        torch.cuda.synchronize()
        ref = alone.to_numpy(ds.dim0, ds.dim1)
        assert np.array_equal(np.ascontiguousarray(j.image).view(np.uint64),
                              np.ascontiguousarray(ref).view(np.uint64)), f"job {j.job_id}"


def test_upload_host_arrays_copies_each_and_checks_destinations(lib):
    """One call, several arrays (page-locked, pageable, device sources, an
    empty one): every destination gets its bytes; a host destination, or a
    host source for the SM-store download, is refused before any copy."""
    rng = np.random.default_rng(9)
    pinned = torch.from_numpy(rng.integers(0, 256, 5000, dtype=np.uint8)).pin_memory()
    plain = rng.integers(0, 256, 777, dtype=np.uint8)
    dev_src = torch.from_numpy(rng.integers(0, 256, 4096, dtype=np.uint8)).cuda()
    sizes = [5000, 777, 4096, 0]
    dsts = [torch.zeros(max(n, 1), dtype=torch.uint8, device="cuda") for n in sizes]
    srcs = [pinned.data_ptr(), plain.ctypes.data, dev_src.data_ptr(), pinned.data_ptr()]
    dp = (C.c_void_p * 4)(*[d.data_ptr() for d in dsts])
    sp = (C.c_void_p * 4)(*srcs)
    nb = (C.c_int64 * 4)(*sizes)
    _lib.check(lib.sarbp_upload_host_arrays(4, dp, sp, nb, _stream()))
    torch.cuda.synchronize()
    assert torch.equal(dsts[0].cpu(), pinned)
    assert np.array_equal(dsts[1].cpu().numpy(), plain)
    assert torch.equal(dsts[2], dev_src)
    assert int(dsts[3].item()) == 0
    host_dst = np.zeros(16, dtype=np.uint8)
    bad = (C.c_void_p * 1)(host_dst.ctypes.data)
    one = (C.c_void_p * 1)(pinned.data_ptr())
    assert lib.sarbp_upload_host_arrays(1, bad, one, (C.c_int64 * 1)(16),
                                        _stream()) == _lib.SARBP_EINVAL
    assert "not device memory" in _lib.last_error()
    out = torch.zeros(16, dtype=torch.uint8).pin_memory()
    assert lib.sarbp_copy_to_host_sm(out.data_ptr(), 0x10, 16, _stream()) == _lib.SARBP_EINVAL


def test_unmapped_host_ranges_are_refused_on_the_host(lib):
    """A host range with an unmapped page in it (or a stray address) is
    refused by the copy entry points before any launch, also on a device
    that reads pageable memory in place (the range is checked on the host
    first)."""
    import mmap as _mmap
    libc = C.CDLL(None, use_errno=True)
    libc.mmap.restype = C.c_void_p
    libc.mmap.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_long]
    libc.munmap.argtypes = [C.c_void_p, C.c_size_t]
    pg = _mmap.PAGESIZE
    base = libc.mmap(None, 3 * pg, _mmap.PROT_READ | _mmap.PROT_WRITE,
                     _mmap.MAP_PRIVATE | _mmap.MAP_ANONYMOUS, -1, 0)
    assert base not in (None, C.c_void_p(-1).value)
    try:
        assert libc.munmap(base + pg, pg) == 0          # a hole in the middle
        dst = torch.zeros(3 * pg, dtype=torch.uint8, device="cuda")
        rc = lib.sarbp_copy_to_device_sm(dst.data_ptr(), base, 3 * pg, _stream())
        assert rc == _lib.SARBP_EINVAL
        rc = lib.sarbp_copy_to_host_sm(base, dst.data_ptr(), 3 * pg, _stream())
        assert rc == _lib.SARBP_EINVAL
        # the mapped first page alone is fine where pageable memory is reachable
        rc = lib.sarbp_copy_to_device_sm(dst.data_ptr(), base, pg, _stream())
        assert rc == (_lib.SARBP_OK if lib.sarbp_device_reads_pageable() else _lib.SARBP_EINVAL)
        torch.cuda.synchronize()
        assert lib.sarbp_copy_to_device_sm(dst.data_ptr(), 0x10, 16,
                                           _stream()) == _lib.SARBP_EINVAL
    finally:
        libc.munmap(base, pg)
        libc.munmap(base + 2 * pg, pg)
