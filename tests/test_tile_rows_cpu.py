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
