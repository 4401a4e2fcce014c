"""Writes the golden fixtures in this directory from the REFERENCE's own code.

Run where the reference tree is available ($MUXI_REF_ROOT, else a
`reference` folder beside this repository's folder; oracle/ref/build_ref.py
finds it the same way):  python tests/golden/make_golden.py

Inputs are seeded synthetic matrices from muxi_spmv_gb300's host generators;
every expected output comes from oracle/_ref/libmuxi_ref.so, i.e. the
reference's functions compiled from its sources by oracle/ref/build_ref.py:
  y_ref_serial   tests/deep_analysis_runner.cpp:184-190 (CPU CSR loop)
  tiles_*        csr5_compute_tile_boundaries_kernel (spmv_csr5.cu:36-58)
  merge_pos      compute_merge_partitions_kernel (spmv_csr5.cu:912-925)
  merge_row/nnz  merge_path_search (spmv_csr5.cu:497-533)
  ell_*          csr_to_ellpack (spmv_ellpack.cu:11-70)
  row_*          reorderMatrixByRowLength (test_row_reordering.cu:99-143)
  com_*          reorderColumns (column_reorder.cuh:42-141)
  sorted_*       sortColumnsWithinRows (column_reorder.cuh:175-201)
  rcm_*, freq_*  reorderColumnsRCM / reorderColumnsByFrequency
                 (test_column_reordering.cu:116-199); their std::sort tie
                 order is unspecified, so only the sort keys are stored for
                 them (the permutation is checked by key order).
The diagonal known-answer case restates tests/correctness/test_spmv.cu:15-30
(A = I, x[i] = i+1, y == x within 1e-5).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import muxi_spmv_gb300 as mx  # noqa: E402
from muxi_spmv_gb300 import workloads as W  # noqa: E402
from oracle import refpin as R  # noqa: E402


def shuffled_rows(rp, ci, v, seed):
    """Same matrix with each row's entries in a seeded random order (input
    for the in-row column sort)."""
    rng = np.random.default_rng(seed)
    c, vv = ci.copy(), v.copy()
    for r in range(len(rp) - 1):
        s, e = rp[r], rp[r + 1]
        p = rng.permutation(e - s)
        c[s:e], vv[s:e] = c[s:e][p], vv[s:e][p]
    return c, vv


def with_empty_rows(rp, ci, v, every):
    """Inserts an empty row after every `every`-th row (adversarial layout)."""
    lens = np.diff(rp)
    out = []
    for r, l in enumerate(lens):
        out.append(l)
        if r % every == 0:
            out.append(0)
    out = np.array(out, np.int32)
    nrp = np.zeros(len(out) + 1, np.int32)
    nrp[1:] = np.cumsum(out)
    return nrp, ci, v


def case(name, rp, ci, v, cols, seed, ell_width=0):
    rows, nnz = len(rp) - 1, len(ci)
    x = mx.gen_vector(cols, W.x_seed(seed))
    d = dict(rowPtr=rp, colIdx=ci, values=v, x=x, numCols=np.int64(cols))
    d["y_ref_serial"] = R.cpu_spmv(rp, ci, v, x)
    for sigma in (128, 256):
        a, b = R.csr5_tiles(rp, nnz, sigma)
        d[f"tiles_row_{sigma}"], d[f"tiles_off_{sigma}"] = a, b
    P = int(mx.lib().spmv_merge_default_partitions(rows, nnz))
    d["merge_P"] = np.int64(P)
    d["merge_pos"] = R.merge_partitions(rows, nnz, P)
    diag = np.arange(0, rows + nnz + 1, max(1, (rows + nnz) // 4000), dtype=np.int32)
    diag = np.unique(np.concatenate([diag, d["merge_pos"], [rows + nnz]])).astype(np.int32)
    d["merge_diag"] = diag
    d["merge_row"], d["merge_nnz"] = R.merge_search(rp, nnz, diag)
    ec, ev, w = R.csr_to_ell(rp, ci, v, cols, ell_width)
    d["ell_col"], d["ell_val"], d["ell_width"] = ec, ev, np.int64(w)
    rm, nrp, nc, nv = R.row_reorder(rp, ci, v, cols)
    d["row_map"], d["row_rowPtr"], d["row_colIdx"], d["row_values"] = rm, nrp, nc, nv
    fm, newc = R.center_of_mass_perm(rp, ci, cols)
    d["com_forward"], d["com_colIdx"] = fm, newc
    sc, sv = shuffled_rows(rp, ci, v, seed + 1)
    d["shuf_colIdx"], d["shuf_values"] = sc, sv
    d["sorted_colIdx"], d["sorted_values"] = R.sort_within_rows(rp, sc, sv, cols)
    perm, _ = R.rcm_perm(rp, ci, cols)
    d["rcm_keys_in_order"] = np.array([_min_row(rp, ci, cols)[c] for c in perm], np.int32)
    perm, _ = R.frequency_perm(rp, ci, cols)
    cnt = np.bincount(ci, minlength=cols).astype(np.int32)
    d["freq_keys_in_order"] = cnt[perm]
    np.savez_compressed(HERE / f"{name}.npz", **d)
    print(name, rows, nnz, "ell width", w)


def _min_row(rp, ci, cols):
    rows = len(rp) - 1
    m = np.full(cols, rows, np.int64)
    rid = np.repeat(np.arange(rows), np.diff(rp))
    np.minimum.at(m, ci, rid)
    return m


def main():
    if not R.available():
        raise SystemExit("reference sources not found; set MUXI_REF_ROOT")
    # Diagonal KAT (tests/correctness/test_spmv.cu:15-30).
    n = 1024
    rp = np.arange(n + 1, dtype=np.int32)
    ci = np.arange(n, dtype=np.int32)
    v = np.ones(n, np.float32)
    x = np.arange(1, n + 1, dtype=np.float32)
    np.savez_compressed(HERE / "kat_diagonal.npz", rowPtr=rp, colIdx=ci, values=v, x=x, y_expected=x.copy(),
                        y_ref_serial=R.cpu_spmv(rp, ci, v, x))
    print("kat_diagonal", n)

    rp, ci, v = mx.generate(W.scaled("poisson16k", 2048, seed=11))
    case("poisson_2k", rp, ci, v, 2048, 11)
    rp, ci, v = mx.generate(W.scaled("powerlaw8m", 3000, seed=12))
    case("powerlaw_3k", rp, ci, v, 3000, 12, ell_width=16)  # truncating ELL width, as the reference allows
    rp, ci, v = mx.generate(W.scaled("stencil2d_4096", 1600, seed=13))
    case("stencil2d_40", rp, ci, v, len(rp) - 1, 13)
    rp, ci, v = mx.generate(W.scaled("powerlaw8m", 1500, seed=14))
    rp, ci, v = with_empty_rows(rp, ci, v, every=3)
    case("empty_rows", rp, ci, v, 1500, 14, ell_width=32)


if __name__ == "__main__":
    main()
