"""Serving: jobs that overlap on the device give the same image as alone.

A Poisson stream of small focusing jobs of different sizes runs through the
continuous-batching engine (jobs admitted while others run, their tiles mixed
in the same persistent launches).  Each job's image must be bit-identical to
the single-scene staged kernel's image of the same inputs, and the HBM budget
must hold.
"""
import numpy as np
import pytest
import torch

from sar_backprojection_gb300 import batch, focus, scene_to_device, serve, synth

pytestmark = pytest.mark.gpu

SIZES = [(128, 32, 2001, 200, 260), (256, 48, 3001, 400, 600), (96, 40, 2401, 900, 1300),
         (160, 64, 4001, 1200, 1600), (64, 32, 2001, 300, 400), (192, 32, 3001, 600, 800)]


@pytest.fixture(scope="module")
def jobs():
    out = []
    arrivals = serve.poisson_arrivals(len(SIZES) * 2, rate_per_s=400.0, seed=3)
    for i in range(len(SIZES) * 2):
        d0, d1, naz, s_lo, s_hi = SIZES[i % len(SIZES)]
        spec = synth.scaled_full(200 + i, d0, d1, naz, s_lo, s_hi)
        sc = synth.generate(spec)                      # host (NumPy) inputs
        out.append(serve.Job(job_id=i, args=synth.focus_args(sc), arrival=float(arrivals[i])))
    return out


def _alone(job, tuning):
    ds = scene_to_device(*job.args, device="cuda")
    res = focus(ds, "mixed", tuning=tuning)
    torch.cuda.synchronize()
    return res.to_numpy(ds.dim0, ds.dim1)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_each_job_same_alone_and_in_the_mix(jobs):
    tuning = batch.staged_tuning()
    eng = serve.ServingEngine(budget_bytes=8 * serve.GB, max_slots=8, wave_items=96,
                              tuning=tuning)
    rep = eng.run(jobs)
    s = rep.summary()
    assert s["completed"] == len(jobs)
    assert s["p99_ms"] >= s["p50_ms"] > 0
    assert rep.peak_bytes <= 8 * serve.GB
    assert rep.waves >= 2
    for j in jobs:
        assert j.image is not None and j.image.shape == j.shape
        assert np.array_equal(_bits(j.image), _bits(_alone(j, tuning))), f"job {j.job_id}"


def test_budget_limits_residency(jobs):
    small = jobs[:4]
    for j in small:
        j.admitted = j.finished = None
        j.image = None
    budget = max(j.nbytes() for j in small) + 1     # one job resident at a time
    eng = serve.ServingEngine(budget_bytes=budget, max_slots=4, wave_items=64)
    rep = eng.run(small)
    assert rep.summary()["completed"] == len(small)
    assert rep.peak_bytes <= budget


def test_fp64_sequential_comparator(jobs):
    r = serve.run_fp64_sequential(jobs[:3])
    assert r["p99_ms"] >= r["p50_ms"] > 0 and r["pixel_pulses"] > 0


def _pinned(args):
    """The same job with page-locked inputs (torch pin_memory), the layout
    the native queue reads by SM loads."""
    out = list(args)
    for i in (0, 1, 2, 3, 4, 8, 12):
        a = np.asarray(args[i])
        out[i] = torch.from_numpy(np.ascontiguousarray(a.T)).pin_memory().t()
    for i in (5, 6, 7):
        out[i] = torch.from_numpy(np.ascontiguousarray(args[i])).pin_memory()
    return tuple(out)


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
def test_native_engine_each_job_same_alone_and_in_the_mix(jobs, memory):
    """The whole request path in the C queue's worker (host inputs in, host
    image out): every job's image equals its single-scene image bit for bit."""
    tuning = batch.staged_tuning()
    mine = [serve.Job(job_id=j.job_id, arrival=j.arrival,
                      args=_pinned(j.args) if memory == "pinned" else j.args) for j in jobs]
    with serve.NativeServingEngine(budget_bytes=8 * serve.GB, max_slots=8, wave_items=96,
                                   tuning=tuning) as eng:
        rep = eng.run(mine)
    s = rep.summary()
    assert s["completed"] == len(jobs) and s["p99_ms"] >= s["p50_ms"] > 0
    for j, ref in zip(mine, jobs):
        assert j.image is not None and j.image.shape == ref.shape
        assert np.array_equal(_bits(j.image), _bits(_alone(ref, tuning))), f"job {j.job_id}"


def test_native_engine_images_meet_the_bars_against_the_oracle(jobs):
    """Served images checked against the oracle directly (not only through
    the single-scene kernel): coherence >= 0.9999, RMS phase <= 1 mrad,
    rel-L2 <= 1e-3, and zero exactly where the oracle has no contributor."""
    from oracle import oracle
    from sar_backprojection_gb300 import quality
    mine = [serve.Job(job_id=j.job_id, arrival=j.arrival, args=j.args) for j in jobs[:6]]
    with serve.NativeServingEngine(budget_bytes=4 * serve.GB, max_slots=4) as eng:
        eng.run(mine)
    for j in mine:
        ref, nv, _ = oracle.focus(*j.args)
        q = quality.compare(j.image, ref)
        assert q["coherence"] >= 0.9999 and q["rms_phase_mrad"] <= 1.0, (j.job_id, q)
        assert q["rel_l2"] <= 1e-3, (j.job_id, q)
        assert (j.image[nv == 0] == 0).all()


def test_native_engine_reserved_memory_limits_residency(jobs):
    """A reserve that holds one job at a time still completes every job; a
    job larger than the whole reserve is refused at submission."""
    small = [serve.Job(job_id=j.job_id, arrival=0.0, args=j.args) for j in jobs[:4]]
    probe = serve.NativeServingEngine(budget_bytes=1 << 30, max_slots=4)
    need = max(probe.job_bytes(j.args) for j in small)
    probe.close()
    with serve.NativeServingEngine(budget_bytes=need, max_slots=4, wave_items=64) as eng:
        rep = eng.run(small)
        assert rep.summary()["completed"] == len(small)
    with serve.NativeServingEngine(budget_bytes=need // 4, max_slots=4) as eng:
        with pytest.raises(Exception) as e:
            eng.run(small[:1], timeout_s=30)
        assert "reserved" in str(e.value)


@pytest.mark.parametrize("reserve", ["arena", "tiny"])
def test_native_engine_resident_jobs_same_alone_and_in_the_mix(jobs, reserve):
    """Device-resident inputs (sarbp_queue_submit) through the native loop:
    each job's chunk-table workspace is carved from the reserved memory (or,
    when the reserve cannot hold it, allocated at admission), and every
    job's image equals its single-scene image bit for bit."""
    tuning = batch.staged_tuning()
    scenes = {j.job_id: scene_to_device(*j.args, device="cuda") for j in jobs}
    mine = [serve.Job(job_id=j.job_id, arrival=j.arrival, args=j.args) for j in jobs]
    budget = 4 * serve.GB if reserve == "arena" else 4096
    with serve.NativeServingEngine(budget_bytes=budget, max_slots=8, wave_items=96,
                                   tuning=tuning) as eng:
        rep = eng.run_resident(mine, lambda j: scenes[j.job_id])
    s = rep.summary()
    assert s["completed"] == len(jobs) and s["h2d_gb"] == 0
    for j, ref in zip(mine, jobs):
        sc = scenes[j.job_id]
        flat = j.image.cpu().numpy().view(np.complex128).reshape(-1)
        img = np.reshape(flat, (sc.dim0, sc.dim1), order="F")
        assert np.array_equal(_bits(img), _bits(_alone(ref, tuning))), f"job {j.job_id}"
