"""Pins the CPU oracle to the reference's own functions, compiled from the
reference sources into oracle/_ref by oracle/ref/build_ref.py, on fresh
seeded inputs.  Needs the reference tree; skipped where it is absent."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

refpin = pytest.importorskip("oracle.refpin")
pytestmark = pytest.mark.refsrc

if not refpin.available():
    pytest.skip("reference sources not present", allow_module_level=True)


def matrices():
    import muxi_spmv_gb300 as mx
    from muxi_spmv_gb300 import workloads as W
    out = []
    for seed, (name, rows) in enumerate([("poisson16k", 700), ("powerlaw8m", 900), ("stencil3d_256", 512),
                                         ("powerlaw8m", 64), ("poisson16k", 1)]):
        s = W.scaled(name, rows, seed=100 + seed)
        rp, ci, v = mx.generate(s)
        out.append((f"{name}-{rows}", rp, ci, v, s.numCols))
    return out


MATS = matrices()


@pytest.mark.parametrize("m", MATS, ids=[m[0] for m in MATS])
def test_pins(m):
    _, rp, ci, v, cols = m
    rows, nnz = len(rp) - 1, len(ci)
    x = np.linspace(-1, 1, cols, dtype=np.float32)
    assert np.array_equal(oracle.cpu_spmv(rp, ci, v, x), refpin.cpu_spmv(rp, ci, v, x))
    for sigma in (64, 128, 256):
        if nnz:
            a, b = oracle.csr5_tiles(rp, nnz, sigma)
            c, d = refpin.csr5_tiles(rp, nnz, sigma)
            assert np.array_equal(a, c) and np.array_equal(b, d)
    for P in (1, 7, oracle.merge_default_partitions(rows, nnz)):
        assert np.array_equal(oracle.merge_partitions(rows, nnz, P), refpin.merge_partitions(rows, nnz, P))
    diag = np.arange(rows + nnz + 1, dtype=np.int32)
    r1, z1 = oracle.merge_search(rp, nnz, diag)
    r2, z2 = refpin.merge_search(rp, nnz, diag)
    assert np.array_equal(r1, r2) and np.array_equal(z1, z2)
    ec, ev, w, _ = oracle.csr_to_ell(rp, ci, v, 0)
    ec2, ev2, w2 = refpin.csr_to_ell(rp, ci, v, cols, 0)
    assert w == w2 and np.array_equal(ec, ec2) and np.array_equal(ev, ev2)
    got = oracle.row_reorder(rp, ci, v)
    want = refpin.row_reorder(rp, ci, v, cols)
    assert all(np.array_equal(p, q) for p, q in zip(got, want))
    fm, _ = oracle.colperm_center_of_mass(rp, ci, cols)
    fm2, newc = refpin.center_of_mass_perm(rp, ci, cols)
    assert np.array_equal(fm, fm2) and np.array_equal(oracle.apply_colperm(fm, ci), newc)
    rng = np.random.default_rng(rows)
    sc, sv = ci.copy(), v.copy()
    for r in range(rows):
        s, e = rp[r], rp[r + 1]
        p = rng.permutation(e - s)
        sc[s:e], sv[s:e] = sc[s:e][p], sv[s:e][p]
    a, b = oracle.sort_within_rows(rp, sc, sv)
    c, d = refpin.sort_within_rows(rp, sc, sv, cols)
    assert np.array_equal(a, c) and np.array_equal(b, d)
    # min-row ("RCM") and frequency: keys in permutation order agree; where a
    # key is unique its position agrees; tie groups hold the same columns.
    for ofn, rfn, keyf in ((lambda: oracle.colperm_min_row(rp, ci, cols), lambda: refpin.rcm_perm(rp, ci, cols),
                            None),
                           (lambda: oracle.colperm_frequency(ci, cols), lambda: refpin.frequency_perm(rp, ci, cols),
                            None)):
        perm, key = ofn()
        perm2, newc2 = rfn()
        assert np.array_equal(key[perm], key[perm2])
        ks = key[perm]
        starts = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]])
        ends = np.r_[starts[1:], len(ks)]
        for s, e in zip(starts, ends):
            assert set(perm[s:e]) == set(perm2[s:e])
        assert np.array_equal(oracle.apply_colperm(perm2, ci), newc2)
