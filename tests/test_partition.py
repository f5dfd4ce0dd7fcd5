"""One scene split by azimuth block across ranks (host logic, oracle, gloo).

Every DEM line must belong to exactly one rank, every pulse a rank's pixels
keep must lie inside that rank's raw window (and be a locally valid pulse),
and a block focused from its own window with re-based pulse indices must
give the whole scene's result on its pixels: the oracle's image and
contributor counts bit for bit.  The two-rank case runs as spawned CPU
processes with the gloo backend; each rank focuses its block with the
oracle and rank 0 assembles the gathered pieces.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import load_golden_scene
from oracle import oracle
from sar_backprojection_gb300 import partition, synth


def _scene_azimuth_on(axis: int, seed: int = 3):
    sc = synth.generate(synth.SceneSpec(name="part", seed=seed, dim0=96, dim1=24, x0=420.0,
                                        naz=1201, nra=512, near_range=3550.0, sint_lo=100,
                                        sint_hi=700, mask_fraction=0.8, terrain_sigma=5.0))
    return synth.azimuth_columns(sc) if axis == 1 else sc


def _kept_pulses(index, sint, mask, naz):
    """Brute force: per pixel (flattened C order) the set of kept pulses."""
    out = []
    for i, s, m in zip(np.ravel(index), np.ravel(sint), np.ravel(mask)):
        if m != 1 or s == -9999:
            out.append(())
            continue
        jj = int(np.ceil(s / 2.0)) * 2 + 1
        off = int(np.ceil(abs(s) / 2.0))
        out.append(tuple(a for a in range(i - off, i - off + jj) if 0 < a < naz - 1))
    return out


def _check_blocks(sc, blocks, axis):
    n = np.shape(sc["xxg1"])[axis]
    naz = sc["RawData"].shape[1]
    covered = np.zeros(n, dtype=int)
    for b in blocks:
        covered[b.line0:b.line1] += 1
        assert b.line0 % 16 == 0 or b.line0 == n
        sl = (slice(b.line0, b.line1), slice(None)) if axis == 0 else \
             (slice(None), slice(b.line0, b.line1))
        kept = _kept_pulses(sc["Index"][sl], sc["Sint"][sl], sc["Mask"][sl], naz)
        allk = [a for k in kept for a in k]
        if allk:
            # inside the window and locally valid (0 < a - pulse0 < pulses - 1)
            assert b.pulse0 < min(allk) and max(allk) < b.pulse1 - 1
            assert b.pulse0 % partition.WINDOW_ALIGN == 0
            assert b.pulse1 % partition.WINDOW_ALIGN == 0 or b.pulse1 == naz
    assert (covered == 1).all()


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("nranks", [1, 2, 3, 5])
def test_blocks_cover_once_and_match_the_whole_scene(axis, nranks):
    sc = _scene_azimuth_on(axis)
    args = synth.focus_args(sc)
    blocks = partition.plan(sc["Index"], sc["Sint"], sc["Mask"], sc["RawData"].shape[1],
                            nranks, axis=axis)
    assert len(blocks) == nranks
    _check_blocks(sc, blocks, axis)
    whole, wnv, _ = oracle.focus_scene(sc)
    imgs, nvs = [], []
    for b in blocks:
        img, nv, _ = oracle.focus(*partition.block_args(args, b))
        imgs.append(img)
        nvs.append(nv.astype(np.complex128))
    assert np.array_equal(partition.assemble(blocks, imgs, whole.shape), whole)
    assert np.array_equal(partition.assemble(blocks, nvs, whole.shape).real, wnv)
    # balanced: each block within one aligned group of lines of its share
    lw = partition.line_work(sc["Index"], sc["Sint"], sc["Mask"], sc["RawData"].shape[1], axis)
    group = max(int(lw[a:a + 16].sum()) for a in range(0, lw.size, 16))
    for b in blocks:
        assert abs(b.work - lw.sum() / nranks) <= group


def test_edge_case_scene_splits_exactly():
    """Apertures at pulses 0, 1, Naz-2, Naz-1, masks 0/1/2, Sint -9999 and
    odd/negative lengths: split along either axis, still the oracle's image."""
    sc, ref = load_golden_scene("edges")
    for axis in (0, 1):
        blocks = partition.plan(sc["Index"], sc["Sint"], sc["Mask"], sc["RawData"].shape[1],
                                2, axis=axis, align=4)
        imgs = [oracle.focus(*partition.block_args(synth.focus_args(sc), b))[0]
                for b in blocks]
        assert np.array_equal(partition.assemble(blocks, imgs, ref.shape), ref)


def test_split_lines_is_balanced_and_aligned():
    work = np.array([0] * 10 + [5] * 90 + [1] * 60)
    cuts = partition.split_lines(work, 4, align=8)
    assert cuts[0][0] == 0 and cuts[-1][1] == work.size
    assert all(a % 8 == 0 for a, _ in cuts)
    assert all(a <= b for a, b in cuts)
    assert [c[1] for c in cuts[:-1]] == [c[0] for c in cuts[1:]]
    # more ranks than aligned lines: trailing ranks get empty blocks
    cuts = partition.split_lines(np.ones(10), 4, align=8)
    assert sum(b - a for a, b in cuts) == 10


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import torch.distributed as dist

    from oracle import oracle as orc
    from sar_backprojection_gb300 import partition as part
    from test_partition import _scene_azimuth_on

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = _scene_azimuth_on(1, seed=9)
    blocks = part.plan(sc["Index"], sc["Sint"], sc["Mask"], sc["RawData"].shape[1], world)
    img, nv, _ = orc.focus(*part.block_args(synth.focus_args(sc), blocks[rank]))
    pieces = [None] * world
    dist.all_gather_object(pieces, (img, nv))      # host gather of the disjoint outputs
    if rank == 0:
        whole, wnv, _ = orc.focus_scene(sc)
        got = part.assemble(blocks, [p[0] for p in pieces], whole.shape)
        gnv = part.assemble(blocks, [p[1].astype(np.complex128) for p in pieces], whole.shape)
        q.put(bool(np.array_equal(got, whole) and np.array_equal(gnv.real, wnv)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_two_gloo_ranks_focus_their_blocks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(150)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True
