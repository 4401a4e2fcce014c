"""The row bookkeeping of the ordered CSR5 tiles with row-start masks
(csr5_tile_rows_bits, tile_bits_kernel), restated in numpy on the golden
matrices that have no empty rows.  The FP32 tiles stage the sums of the rows
they complete and store them in one coalesced pass; that relies on the rows
a tile completes being rFirst, rFirst + 1, ... with their count equal to the
row starts inside the tile plus one when the tile's last row ends at the tile
end.  CPU only."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"


def row_start_masks(rowPtr, nnz, sigma):
    """Per tile: the set positions k >= 1 where a row starts, and whether the
    tile's last row ends exactly at the tile end (bit 0 of word 0)."""
    tiles = (nnz + sigma - 1) // sigma
    starts = [set() for _ in range(tiles)]
    ends_at_end = np.zeros(tiles, bool)
    ends_at_end[tiles - 1] = True  # the last tile's last row ends at its end
    for r in range(1, len(rowPtr) - 1):
        pos = int(rowPtr[r])
        t, k = divmod(pos, sigma)
        if k:
            starts[t].add(k)
        else:
            ends_at_end[t - 1] = True
    return starts, ends_at_end


@pytest.mark.parametrize("name", ["poisson_2k", "powerlaw_3k", "stencil2d_40"])
@pytest.mark.parametrize("sigma", [128, 256, 512])
def test_completed_rows_are_consecutive_from_first_row(name, sigma):
    g = dict(np.load(GOLD / f"{name}.npz"))
    rp = g["rowPtr"].astype(np.int64)
    nnz = int(rp[-1])
    assert (np.diff(rp) > 0).all()  # the masks are built only for matrices without empty rows
    tile_row, _ = oracle.csr5_tiles(g["rowPtr"], nnz, sigma)
    starts, ends_at_end = row_start_masks(rp, nnz, sigma)
    last = rp[1:] - 1  # position of each row's last nonzero
    for t in range(len(tile_row)):
        t0, t1 = t * sigma, min(t * sigma + sigma, nnz)
        completed = np.nonzero((last >= t0) & (last < t1))[0]
        n = len(starts[t]) + int(ends_at_end[t])
        assert np.array_equal(completed, np.arange(tile_row[t], tile_row[t] + n)), (name, sigma, t)
        assert n <= sigma  # the staging region holds at least 32*E = sigma values


def kogge_stone_segmented(keys, vals, max_steps=None):
    """The warp scan of the tile row logic, lane by lane: step `off` adds the
    value of lane - off when that lane has the same key."""
    v = np.array(vals, dtype=np.float64)
    off, steps = 1, 0
    while off < 32 and (max_steps is None or steps < max_steps):
        prev = v.copy()
        for lane in range(off, 32):
            if keys[lane - off] == keys[lane]:
                v[lane] = prev[lane] + prev[lane - off]
        off <<= 1
        steps += 1
    return v


def test_segmented_scan_stops_at_longest_key_run():
    """key_run_length: with keys rising over the lanes, the steps whose offset
    is below the longest run of equal keys already give the full scan (the
    FP64 tiles skip the rest)."""
    rng = np.random.default_rng(3)
    for _ in range(2000):
        run_cap = int(rng.integers(1, 33))
        lens = []
        while sum(lens) < 32:
            lens.append(int(rng.integers(1, run_cap + 1)))
        keys = np.repeat(np.arange(len(lens)), lens)[:32]
        if rng.random() < 0.2:  # lanes without elements carry the largest key at the end
            keys[32 - int(rng.integers(1, 16)):] = 0x7FFFFFFF
        vals = rng.integers(-1000, 1000, 32).astype(np.float64)  # exact sums
        span = max(int(np.sum(keys[: l + 1] == keys[l])) for l in range(32))
        steps = 0
        while (1 << steps) < span:
            steps += 1
        full = kogge_stone_segmented(keys, vals)
        short = kogge_stone_segmented(keys, vals, max_steps=steps)
        assert np.array_equal(full, short), (keys, span)
        # and the full scan is the segmented inclusive prefix sum
        ref = np.array([vals[: l + 1][keys[: l + 1] == keys[l]].sum() for l in range(32)])
        assert np.array_equal(full, ref)
