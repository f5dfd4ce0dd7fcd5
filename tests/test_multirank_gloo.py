"""bench.py's host logic on CPU: the multi-rank bookkeeping (two gloo ranks,
one scene each) and the autotuner's choice among timed candidates.

The focusing path shards by scene (weak scaling, no collective on the data
path); the only cross-rank operations are the barrier around the timed
region and the max-over-ranks of the step time.  Ranks here run as spawned
CPU processes with the gloo backend (rendezvous on 127.0.0.1).
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench
    from sar_backprojection_gb300 import synth

    d = bench.Dist()
    d.init("gloo")
    spec, name = bench.workload_spec(type("A", (), {"workload": "full", "seed": 2})(), d.rank)
    d.barrier()
    t = d.max(10.0 + rank, "cpu")
    d.barrier()
    q.put((rank, spec.seed, t, name))
    d.close()


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(90)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[0] for r in res] == [0, 1]
    assert res[0][1] != res[1][1]               # one distinct scene per rank
    assert res[0][2] == res[1][2] == 11.0       # max over ranks


def test_autotuner_prefers_earlier_candidates_within_noise():
    import bench
    # 208-bin window listed first: kept when a later candidate wins by < 1 %
    assert bench.choose_tuning([(1.7174, "w208"), (1.7681, "c64"), (1.7161, "w192")]) == "w208"
    assert bench.choose_tuning([(1.80, "w208"), (1.70, "w192")]) == "w192"
    assert bench.choose_tuning([(2.0, "a")]) == "a"
