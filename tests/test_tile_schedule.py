"""The launch schedule of the paired TMA backprojection's half-tile tail
(gather_rot.cu: gather_rot_tma on the host, k_gather_rot_tma's tile
mapping), restated on the CPU.

T = gx * gy uniform tiles over S SMs: when T > S and T mod S != 0, the last
T mod S tiles run as half tiles, two CTAs each, in a grid of gx columns and
ceil((nfull + 2 nhalf) / gx) rows; CTAs past nfull + 2 nhalf return at once.
Every tile must be summed exactly once, whole or as its two halves (part 0:
the rows of warps 0-3, part 1: those of warps 4-7), so that each pixel gets
exactly one partial sum from its tile (and one from its quarter-turned
tile's CTA).
"""
import collections

import pytest


def schedule(gx, gy, sms):
    """(grid rows, nfull, nhalf) as the host computes them."""
    T = gx * gy
    if sms > 0 and T > sms and T % sms:
        nhalf = T % sms
        nfull = T - nhalf
        return (nfull + 2 * nhalf + gx - 1) // gx, nfull, nhalf
    return gy, 0, 0


def cta_tile(bx, by, gx, nfull, nhalf):
    """The kernel's mapping of CTA (bx, by) to (tx, ty, part), or None for a
    spare CTA of the grid's last row."""
    if nhalf == 0:
        return bx, by, -1
    t = by * gx + bx
    part = -1
    if t >= nfull:
        h = t - nfull
        if h >= 2 * nhalf:
            return None
        t = nfull + (h >> 1)
        part = h & 1
    return t % gx, t // gx, part


@pytest.mark.parametrize("gx,gy", [(64, 32), (32, 16), (25, 13), (7, 3), (152, 1), (153, 1),
                                   (1, 400), (48, 24), (64, 64)])
@pytest.mark.parametrize("sms", [152, 148, 132, 1])
def test_every_tile_once_whole_or_as_two_halves(gx, gy, sms):
    rows, nfull, nhalf = schedule(gx, gy, sms)
    seen = collections.defaultdict(list)
    for by in range(rows):
        for bx in range(gx):
            m = cta_tile(bx, by, gx, nfull, nhalf)
            if m is None:
                continue
            tx, ty, part = m
            assert 0 <= tx < gx and 0 <= ty < gy
            seen[(tx, ty)].append(part)
    assert len(seen) == gx * gy
    halves = 0
    for parts in seen.values():
        assert sorted(parts) in ([-1], [0, 1])
        halves += parts != [-1]
    assert halves == nhalf
    # the whole tiles come first in launch order, then the halves
    if nhalf:
        assert nfull % sms == 0 or sms == 1


def test_benchmark_shape():
    """2048^2 with 8-row tiles on 152 SMs: 2048 tiles, the last 72 in
    halves, a grid of 34 rows of 64 CTAs (56 spare)."""
    rows, nfull, nhalf = schedule(64, 32, 152)
    assert (rows, nfull, nhalf) == (34, 1976, 72)
    assert rows * 64 - (nfull + 2 * nhalf) == 56
