"""One scene split across GPUs by azimuth block.

The reference scales to large scenes by walking the DEM in azimuth batches
and giving each batch only the raw-data azimuth window its apertures reach,
with pulse indices made relative to that window (main_gpu.py:415-417,
:465-494, chunk-relative indexing in its kernel K2, :60-155).  The same cut
splits one scene across devices: every pixel is independent and only reads
raw data, so each rank focuses a contiguous block of azimuth lines of the
DEM from its own HBM copy of its pulse window, and the blocks' images are
disjoint pieces of the whole image -- no collective on the data path, no
peer-memory loads; the host concatenates the pieces.

Blocks are balanced by nominal work (the kept aperture lengths of their
pixels) and start on multiples of ``align`` lines (the pixel-tile extent),
so each rank's tiles are the whole scene's tiles.  A rank's pulse window is
widened to multiples of ``WINDOW_ALIGN`` pulses (the longest chunk of the
mixed kernels, a multiple of both stage lengths): its chunk references, pulse
tables and stage windows are then those of the whole scene, and the mixed
kernel's image of a block equals the whole scene's image on those pixels bit
for bit.  Pulse validity stays the reference's global rule 0 < a < Naz-1
(sar_focuser_puntual_noui.py:46-55): a window never ends on a pulse some
pixel keeps, so the local bound drops no kept pulse and admits no pulse the
global bound rejects.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

WINDOW_ALIGN = 128


@dataclass(frozen=True)
class Block:
    """One rank's share of a scene: DEM lines [line0, line1) along ``axis``
    and raw pulses [pulse0, pulse1) (pulse1 - pulse0 pulses, local pulse p is
    global pulse pulse0 + p)."""

    rank: int
    axis: int
    line0: int
    line1: int
    pulse0: int
    pulse1: int
    work: int            # nominal pixel-pulses of the block

    @property
    def lines(self) -> int:
        return self.line1 - self.line0

    @property
    def pulses(self) -> int:
        return self.pulse1 - self.pulse0


def _aperture(index, sint, mask, naz):
    """Per pixel: kept flag, first and last kept pulse, nominal length."""
    s = np.asarray(sint, dtype=np.int64)
    idx = np.asarray(index, dtype=np.int64)
    m = np.asarray(mask).astype(np.uint8)
    half = np.where(s >= 0, (s + 1) // 2, -((-s) // 2))
    jj = half * 2 + 1                                  # ceil(s/2)*2 + 1
    off = (np.abs(s) + 1) // 2                         # ceil(|s|/2)
    ok = (m == 1) & (s != -9999) & (jj > 0)
    lo = np.maximum(idx - off, 1)
    hi = np.minimum(idx - off + jj - 1, naz - 2)
    kept = ok & (lo <= hi)
    return kept, lo, hi, np.where(ok, jj, 0)


def line_work(index, sint, mask, naz: int, axis: int) -> np.ndarray:
    """Nominal pixel-pulses of every DEM line along ``axis``."""
    _, _, _, jj = _aperture(index, sint, mask, naz)
    return jj.sum(axis=1 - axis)


def split_lines(work: np.ndarray, nranks: int, align: int = 16) -> list[tuple[int, int]]:
    """Contiguous [start, end) line ranges, one per rank, with starts on
    multiples of ``align``, balancing the summed work (greedy on the prefix
    sum: each cut at the aligned line nearest the ideal share)."""
    n = int(work.size)
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    csum = np.concatenate([[0], np.cumsum(work, dtype=np.int64)])
    total = int(csum[-1])
    cuts = [0]
    for r in range(1, nranks):
        target = total * r / nranks
        cand = np.arange(cuts[-1], n + 1, align)
        if cand.size == 0 or cand[-1] != n:
            cand = np.append(cand, n)
        c = int(cand[np.argmin(np.abs(csum[cand] - target))])
        cuts.append(max(c, cuts[-1]))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(nranks)]


def pulse_window(index, sint, mask, naz: int) -> tuple[int, int]:
    """[pulse0, pulse1) of raw pulses a block needs: the kept pulses' hull
    plus one pulse each side, widened to multiples of WINDOW_ALIGN (the end
    clamped to Naz); (0, 0) when the block keeps no pulse."""
    kept, lo, hi, _ = _aperture(index, sint, mask, naz)
    if not kept.any():
        return 0, 0
    first, last = int(lo[kept].min()), int(hi[kept].max())
    p0 = ((first - 1) // WINDOW_ALIGN) * WINDOW_ALIGN
    p1 = min(naz, -(-(last + 2) // WINDOW_ALIGN) * WINDOW_ALIGN)
    return p0, p1


def plan(index, sint, mask, naz: int, nranks: int, axis: int = 1,
         align: int = 16) -> list[Block]:
    """Azimuth blocks of a scene for ``nranks`` ranks (``axis``: the DEM axis
    along which azimuth runs -- 1 in the reference's large-scene layout
    (DimRg, DimAz), main_gpu.py:321-324)."""
    if axis not in (0, 1):
        raise ValueError("axis must be 0 or 1")
    index = np.asarray(index)
    work = line_work(index, sint, mask, naz, axis)
    blocks = []
    for r, (a, b) in enumerate(split_lines(work, nranks, align)):
        sl = (slice(a, b), slice(None)) if axis == 0 else (slice(None), slice(a, b))
        p0, p1 = pulse_window(index[sl], np.asarray(sint)[sl], np.asarray(mask)[sl], naz)
        blocks.append(Block(rank=r, axis=axis, line0=a, line1=b, pulse0=p0, pulse1=p1,
                            work=int(work[a:b].sum())))
    return blocks


def block_args(args: tuple, blk: Block) -> tuple:
    """The 13 focusing arguments of one block: its DEM lines, Index made
    relative to the pulse window, the window's trajectory and raw pulses.
    Host arrays (NumPy or memory maps) are sliced, never copied whole."""
    (xxg1, yyg1, zzg1, mask, index, wgsx, wgsy, wgsz, raw, near, dra, lam, sint) = args
    sl = ((slice(blk.line0, blk.line1), slice(None)) if blk.axis == 0
          else (slice(None), slice(blk.line0, blk.line1)))

    def grid(a):
        return np.asfortranarray(np.asarray(a)[sl])

    p0, p1 = blk.pulse0, max(blk.pulse1, blk.pulse0 + 1)
    idx = np.asarray(index)[sl].astype(np.int64) - p0
    idx = np.asfortranarray(np.clip(idx, np.iinfo(np.int32).min, np.iinfo(np.int32).max)
                            .astype(np.int32))
    traj = [np.ascontiguousarray(np.asarray(w)[p0:p1], dtype=np.float64)
            for w in (wgsx, wgsy, wgsz)]
    if hasattr(raw, "detach"):
        rawb = raw[:, p0:p1]
    else:
        rawb = np.asarray(raw)[:, p0:p1]
    return (grid(xxg1), grid(yyg1), grid(zzg1), grid(mask), idx, traj[0], traj[1], traj[2],
            rawb, near, dra, lam, grid(sint))


def assemble(blocks: list[Block], images: list[np.ndarray], shape: tuple[int, int]) -> np.ndarray:
    """The whole complex128 image from the blocks' images (column-major)."""
    out = np.zeros(shape, dtype=np.complex128, order="F")
    for blk, img in zip(blocks, images):
        if blk.axis == 0:
            out[blk.line0:blk.line1, :] = img
        else:
            out[:, blk.line0:blk.line1] = img
    return out


def focus_block(args: tuple, blocks: list[Block], rank: int, **kw) -> np.ndarray:
    """Focus this rank's block on the current device through the drop-in call
    (keyword arguments pass through: precision, tuning, device)."""
    from .focuser import FocalizzatoreBpPx

    blk = blocks[rank]
    if blk.lines == 0:
        shape = (0, np.shape(args[0])[1]) if blk.axis == 0 else (np.shape(args[0])[0], 0)
        return np.zeros(shape, dtype=np.complex128, order="F")
    if blk.pulses == 0:        # nothing kept: the image is zero
        a = block_args(args, blk)
        return np.zeros(np.shape(a[0]), dtype=np.complex128, order="F")
    return FocalizzatoreBpPx(*block_args(args, blk), **kw)
