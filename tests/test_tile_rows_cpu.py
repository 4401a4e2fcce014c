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


def swizzled_word(f: int) -> int:
    """Stored position of 16-byte word f of an FP32 product hand-off
    (csr5_ordered.cuh: swizzled_word)."""
    return f ^ ((f >> 3) & 7)


@pytest.mark.parametrize("E", [4, 8, 16])
def test_fp32_handoff_swizzle_is_conflict_free(E):
    """FP32 tiles write product j = lane + 32e (nonzero order) into word j/4,
    component j%4, of a swizzled layout and read a lane's E consecutive
    products back as E/4 16-byte words.  The layout must be a permutation of
    the 8E words, each write instruction must hit all 32 banks once, and each
    eight-lane phase of a 16-byte read must touch eight distinct 16-byte bank
    groups (no bank conflicts either way)."""
    words = 8 * E
    assert sorted(swizzled_word(f) for f in range(words)) == list(range(words))
    for e in range(E):
        banks = {(4 * swizzled_word((lane + 32 * e) >> 2) + ((lane + 32 * e) & 3)) % 32 for lane in range(32)}
        assert len(banks) == 32
    for q in range(E // 4):
        for phase in range(4):
            groups = {swizzled_word(lane * (E // 4) + q) % 8 for lane in range(8 * phase, 8 * phase + 8)}
            assert len(groups) == 8
    # lane l's words hold its products l*E .. l*E + E - 1 in order
    store = {}
    for lane in range(32):
        for e in range(E):
            j = lane + 32 * e
            store[4 * swizzled_word(j >> 2) + (j & 3)] = j
    for lane in range(32):
        got = [store[4 * swizzled_word(lane * (E // 4) + q) + c] for q in range(E // 4) for c in range(4)]
        assert got == list(range(lane * E, lane * E + E))
