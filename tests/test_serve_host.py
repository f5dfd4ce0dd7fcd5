"""Host logic of the serving engine (no GPU): arrivals, sizing, wave policy."""
from types import SimpleNamespace

import numpy as np
import pytest

from sar_backprojection_gb300 import serve


def test_poisson_arrivals():
    t = serve.poisson_arrivals(20000, rate_per_s=50.0, seed=1)
    assert np.all(np.diff(t) > 0)
    assert abs(np.mean(np.diff(t)) - 1 / 50.0) < 1e-3
    assert np.array_equal(t, serve.poisson_arrivals(20000, 50.0, seed=1))


def test_job_bytes_counts_raw_and_padding():
    b = serve.job_bytes(4000, 250, 4762, 40001)
    assert 8 * 4762 * 40001 < b < 8 * 4762 * 40001 + 200 * 10**6
    assert serve.job_bytes(10, 10, 5, 10) >= 8 * 6 * 10       # odd Nra padded


def _fake_engine(policy, wave_items):
    eng = serve.ServingEngine.__new__(serve.ServingEngine)
    eng.policy = policy
    eng.wave_items = wave_items
    return eng


def _active(arrival, ntiles):
    return SimpleNamespace(job=SimpleNamespace(arrival=arrival), ntiles=ntiles, next_tile=0)


def test_wave_fifo_fills_from_oldest_job():
    eng = _fake_engine("fifo", 5)
    a, b = _active(1.0, 3), _active(0.5, 4)
    wave = eng._build_wave([a, b])
    assert [(x is b, t0, t1) for x, t0, t1 in wave] == [(True, 0, 4), (False, 0, 1)]
    assert b.next_tile == 4 and a.next_tile == 1
    assert eng._build_wave([a, b]) == [(a, 1, 3)]


def test_wave_srpt_prefers_short_jobs():
    eng = _fake_engine("srpt", 4)
    a, b = _active(0.0, 10), _active(5.0, 2)
    wave = eng._build_wave([a, b])
    assert [(x is b, t0, t1) for x, t0, t1 in wave] == [(True, 0, 2), (False, 0, 2)]


def test_summary_percentiles():
    jobs = [SimpleNamespace(latency=v / 1e3, nominal=100) for v in range(1, 101)]
    rep = serve.ServingReport(jobs=jobs, wall_s=2.0, waves=3, gpu_launches=9,
                              peak_bytes=serve.GB)
    s = rep.summary()
    assert s["p50_ms"] == pytest.approx(50.5) and s["p99_ms"] == pytest.approx(99.01)
    assert s["pixel_pulses"] == 10000 and s["peak_resident_gb"] == 1.0


def test_batch_item_orders():
    """Work-queue orders of the batch kernel: decreasing cost, decreasing cost
    class with the natural tile order inside a class, natural."""
    import torch
    from sar_backprojection_gb300.batch import item_order
    c = torch.tensor([5, 1, 9, 9, 2, 8, 0])
    assert item_order(c, "cost").tolist() == [2, 3, 5, 0, 4, 1, 6]
    assert item_order(c, "bucket", buckets=4).tolist() == [2, 3, 5, 0, 1, 4, 6]
    assert item_order(c, "natural").tolist() == list(range(7))
    assert item_order(torch.tensor([], dtype=torch.int64), "bucket").numel() == 0
