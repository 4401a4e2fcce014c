"""The CPU oracle against the golden fixtures (outputs of the reference's own
code, tests/golden/make_golden.py) and the reference's known-answer test.
CPU only."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"
CASES = ["poisson_2k", "powerlaw_3k", "stencil2d_40", "empty_rows"]


def load(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def test_kat_diagonal():
    """tests/correctness/test_spmv.cu:15-42: A = I, x[i] = i+1, |y - x| <= 1e-5."""
    g = load("kat_diagonal")
    y, a = oracle.spmv_ref(g["rowPtr"], g["colIdx"], g["values"], g["x"])
    assert np.max(np.abs(y - g["y_expected"])) <= 1e-5
    assert np.array_equal(oracle.cpu_spmv(g["rowPtr"], g["colIdx"], g["values"], g["x"]), g["y_ref_serial"])


@pytest.mark.parametrize("name", CASES)
def test_cpu_loop_matches_reference_loop(name):
    """The restated serial loop is bit-identical to the reference's
    (deep_analysis_runner.cpp:184-190), serial and row-parallel."""
    g = load(name)
    for threads in (1, 3):
        y = oracle.cpu_spmv(g["rowPtr"], g["colIdx"], g["values"], g["x"], threads=threads)
        assert np.array_equal(y, g["y_ref_serial"])


@pytest.mark.parametrize("name", CASES)
def test_fp64_oracle_bounds_reference_loop(name):
    """The FP32 reference loop lies within the FP32 bound of the FP64 oracle."""
    g = load(name)
    y, a = oracle.spmv_ref(g["rowPtr"], g["colIdx"], g["values"], g["x"])
    assert np.all(oracle.row_errors(g["y_ref_serial"], y, a, 1e-5) <= 1.0)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("sigma", [128, 256])
def test_csr5_tiles(name, sigma):
    g = load(name)
    a, b = oracle.csr5_tiles(g["rowPtr"], len(g["colIdx"]), sigma)
    assert np.array_equal(a, g[f"tiles_row_{sigma}"])
    assert np.array_equal(b, g[f"tiles_off_{sigma}"])


@pytest.mark.parametrize("name", CASES)
def test_merge_partitions_and_search(name):
    g = load(name)
    rows, nnz = len(g["rowPtr"]) - 1, len(g["colIdx"])
    P = int(g["merge_P"])
    assert oracle.merge_default_partitions(rows, nnz) == P
    assert np.array_equal(oracle.merge_partitions(rows, nnz, P), g["merge_pos"])
    r, z = oracle.merge_search(g["rowPtr"], nnz, g["merge_diag"])
    assert np.array_equal(r, g["merge_row"]) and np.array_equal(z, g["merge_nnz"])


@pytest.mark.parametrize("name", CASES)
def test_ell(name):
    g = load(name)
    ec, ev, w, trunc = oracle.csr_to_ell(g["rowPtr"], g["colIdx"], g["values"], int(g["ell_width"]))
    assert w == int(g["ell_width"])
    assert np.array_equal(ec, g["ell_col"]) and np.array_equal(ev, g["ell_val"])


@pytest.mark.parametrize("name", CASES)
def test_row_reorder(name):
    g = load(name)
    rm, nrp, nc, nv = oracle.row_reorder(g["rowPtr"], g["colIdx"], g["values"])
    assert np.array_equal(rm, g["row_map"]) and np.array_equal(nrp, g["row_rowPtr"])
    assert np.array_equal(nc, g["row_colIdx"]) and np.array_equal(nv, g["row_values"])


@pytest.mark.parametrize("name", CASES)
def test_center_of_mass(name):
    g = load(name)
    fm, key = oracle.colperm_center_of_mass(g["rowPtr"], g["colIdx"], int(g["numCols"]))
    assert np.array_equal(fm, g["com_forward"])
    # column_reorder.cuh:95-112 remaps colIdx with the inverse (old -> new).
    assert np.array_equal(oracle.apply_colperm(fm, g["colIdx"]), g["com_colIdx"])


@pytest.mark.parametrize("name", CASES)
def test_sort_within_rows(name):
    g = load(name)
    c, v = oracle.sort_within_rows(g["rowPtr"], g["shuf_colIdx"], g["shuf_values"])
    assert np.array_equal(c, g["sorted_colIdx"]) and np.array_equal(v, g["sorted_values"])


@pytest.mark.parametrize("name", CASES)
def test_min_row_and_frequency_keys(name):
    """std::sort ties are unspecified in the reference; the key sequence in
    permutation order is what both must agree on."""
    g = load(name)
    cols = int(g["numCols"])
    perm, key = oracle.colperm_min_row(g["rowPtr"], g["colIdx"], cols)
    assert np.array_equal(key[perm], g["rcm_keys_in_order"])
    perm, key = oracle.colperm_frequency(g["colIdx"], cols)
    assert np.array_equal(key[perm], g["freq_keys_in_order"])


def test_merge_search_properties():
    """Every diagonal maps to the unique (row, nnz) with row+nnz = k and
    rowPtr[row] <= nnz <= rowPtr[row+1] (brute force)."""
    g = load("empty_rows")
    rp = g["rowPtr"].astype(np.int64)
    rows, nnz = len(rp) - 1, int(rp[-1])
    diag = np.arange(rows + nnz + 1, dtype=np.int32)
    r, z = oracle.merge_search(g["rowPtr"], nnz, diag)
    assert np.all(r.astype(np.int64) + z == diag)
    assert np.all(rp[r] <= z)
    ok_hi = np.where(r < rows, z <= rp[np.minimum(r + 1, rows)], True)
    assert np.all(ok_hi)
