"""GPU format conversion and reordering: index outputs bit-exact against the
golden fixtures (made by the reference's own code) and the CPU oracle; CSR5 /
ELL SpMV within the FP32/FP64 row bounds of the FP64 oracle."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
NAMES = ["poisson_2k", "powerlaw_3k", "stencil2d_40", "empty_rows"]


def gold(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def gA(mx, g, dtype=np.float32):
    return device_csr(mx, g["rowPtr"], g["colIdx"], g["values"].astype(dtype), int(g["numCols"]))


def host(t):
    return t.cpu().numpy()


def check_y(y, y0, rp, ci, v, xh, alpha, beta):
    yr, a = oracle.spmv_ref(rp, ci, v, xh)
    want = alpha * yr + (beta * y0.astype(np.float64) if beta != 0 else 0.0)
    scale = abs(alpha) * a + (abs(beta) * np.abs(y0.astype(np.float64)) if beta != 0 else 0.0)
    eps = np.finfo(v.dtype).eps
    err = np.abs(host(y).astype(np.float64) - want)
    # the epilogue's rounding of alpha*s + beta*y only when there is one
    slack = 2 * eps * np.abs(want) if (alpha != 1.0 or beta != 0.0) else 0.0
    bad = np.flatnonzero(err > tol_for(v.dtype) * scale + slack)
    assert bad.size == 0, (bad[:5], err[bad[:5]])


@pytest.mark.parametrize("name", NAMES)
def test_csr5_tiles_golden(mx, cuda, name):
    g = gold(name)
    A = gA(mx, g)
    for sigma in (128, 256):
        m = mx.csr5_preprocess(A, sigma=sigma)
        assert np.array_equal(host(m.d_tile_row_ptr)[: m.numTiles], g[f"tiles_row_{sigma}"])
        assert np.array_equal(host(m.d_tile_nnz_offset)[: m.numTiles], g[f"tiles_off_{sigma}"])
    assert mx.csr5_preprocess(A).sigma == 128  # getCSR5Config for warp 32


@pytest.mark.parametrize("name", NAMES)
def test_ell_golden(mx, cuda, name):
    g = gold(name)
    A = gA(mx, g)
    W = int(g["ell_width"])
    e = mx.csr_to_ellpack(A, maxElements=W)
    n = A.numRows * W
    assert np.array_equal(host(e.d_colIdx)[:n], g["ell_col"])
    assert np.array_equal(host(e.d_values)[:n], g["ell_val"])
    _, _, _, trunc = oracle.csr_to_ell(g["rowPtr"], g["colIdx"], g["values"], W)
    assert e.truncatedRows == trunc
    assert mx.max_row_length(A) == oracle.lib().oracle_max_row_length(A.numRows, A.rowPtr.ctypes.data_as(
        __import__("ctypes").c_void_p))


@pytest.mark.parametrize("name", NAMES)
def test_row_reorder_golden(mx, cuda, name):
    torch = cuda
    g = gold(name)
    A = gA(mx, g)
    rm, B = mx.reorder_rows_by_length(A)
    assert np.array_equal(host(rm), g["row_map"])
    assert np.array_equal(host(B.d_rowPtr), g["row_rowPtr"])
    assert np.array_equal(host(B.d_colIdx)[: A.nnz], g["row_colIdx"])
    assert np.array_equal(host(B.d_values)[: A.nnz], g["row_values"])
    # SpMV on the reordered matrix, scattered back, equals the oracle on the original.
    x = torch.from_numpy(g["x"]).cuda()
    B.nnz = A.nnz
    yp = torch.empty(A.numRows, device="cuda")
    mx.spmv_csr(B, x, yp)
    y = torch.empty_like(yp)
    mx.restore_order(yp, rm, y)
    torch.cuda.synchronize()
    check_y(y, np.zeros(A.numRows, np.float32), g["rowPtr"], g["colIdx"], g["values"], g["x"], 1.0, 0.0)
    assert np.array_equal(host(y), oracle.restore_order(host(yp), host(rm)))


@pytest.mark.parametrize("name", NAMES)
def test_column_orders_golden(mx, cuda, name):
    g = gold(name)
    A = gA(mx, g)
    cols = int(g["numCols"])
    perm, key = mx.column_perm(A, mx.COLPERM_CENTER_OF_MASS)
    assert np.array_equal(host(perm), g["com_forward"])
    assert np.array_equal(host(mx.apply_column_perm(A, perm)), g["com_colIdx"])
    _, okey = oracle.colperm_center_of_mass(g["rowPtr"], g["colIdx"], cols)
    assert np.array_equal(host(key).view(np.uint32), okey.view(np.uint32))
    perm, key = mx.column_perm(A, mx.COLPERM_MIN_ROW)
    operm, okey = oracle.colperm_min_row(g["rowPtr"], g["colIdx"], cols)
    assert np.array_equal(host(perm), operm) and np.array_equal(host(key), okey)
    assert np.array_equal(okey[host(perm)], g["rcm_keys_in_order"])
    perm, key = mx.column_perm(A, mx.COLPERM_FREQUENCY)
    operm, okey = oracle.colperm_frequency(g["colIdx"], cols)
    assert np.array_equal(host(perm), operm) and np.array_equal(host(key), okey)
    assert np.array_equal(okey[host(perm)], g["freq_keys_in_order"])
    x = cuda.from_numpy(g["x"]).cuda()
    assert np.array_equal(host(mx.permute_x(perm, x)), oracle.permute_x(operm, g["x"]))


@pytest.mark.parametrize("name", NAMES)
def test_sort_within_rows_golden(mx, cuda, name):
    g = gold(name)
    A = device_csr(mx, g["rowPtr"], g["shuf_colIdx"], g["shuf_values"], int(g["numCols"]))
    mx.sort_columns_within_rows(A)
    assert np.array_equal(host(A.d_colIdx)[: A.nnz], g["sorted_colIdx"])
    assert np.array_equal(host(A.d_values)[: A.nnz], g["sorted_values"])


def test_sort_within_rows_duplicates_and_f64(mx, cuda):
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 40, 500).astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = rng.integers(0, 12, rp[-1]).astype(np.int32)  # many duplicate columns per row
    v = rng.choice([-2.0, -0.5, 0.5, 3.0], rp[-1]).astype(np.float32)
    c2, v2 = oracle.sort_within_rows(rp, ci, v)
    A = device_csr(mx, rp, ci, v, 12)
    mx.sort_columns_within_rows(A)
    assert np.array_equal(host(A.d_colIdx)[: A.nnz], c2) and np.array_equal(host(A.d_values)[: A.nnz], v2)
    A = device_csr(mx, rp, ci, v.astype(np.float64), 12)
    mx.sort_columns_within_rows(A)
    assert np.array_equal(host(A.d_colIdx)[: A.nnz], c2)
    assert np.array_equal(host(A.d_values)[: A.nnz], v2.astype(np.float64))


def larger_cases(mx):
    from muxi_spmv_gb300 import workloads as W
    out = []
    for name, rows, seed in (("powerlaw8m", 80000, 21), ("poisson16k", 16384, 0), ("stencil3d_256", 24 ** 3, 22)):
        s = W.scaled(name, rows, seed) if name != "poisson16k" else W.spec(name)
        out.append((name, *mx.generate(s), s.numCols))
    return out


def test_preprocess_matches_oracle_larger(mx, cuda):
    for name, rp, ci, v, cols in larger_cases(mx):
        A = device_csr(mx, rp, ci, v, cols)
        m = mx.csr5_preprocess(A, sigma=128)
        a, b = oracle.csr5_tiles(rp, len(ci), 128)
        assert np.array_equal(host(m.d_tile_row_ptr), a) and np.array_equal(host(m.d_tile_nnz_offset), b)
        rm, B = mx.reorder_rows_by_length(A)
        orm, onrp, onc, onv = oracle.row_reorder(rp, ci, v)
        assert np.array_equal(host(rm), orm) and np.array_equal(host(B.d_rowPtr), onrp)
        assert np.array_equal(host(B.d_colIdx)[: len(ci)], onc)
        perm, _ = mx.column_perm(A, mx.COLPERM_CENTER_OF_MASS)
        assert np.array_equal(host(perm), oracle.colperm_center_of_mass(rp, ci, cols)[0])
        perm, _ = mx.column_perm(A, mx.COLPERM_MIN_ROW)
        assert np.array_equal(host(perm), oracle.colperm_min_row(rp, ci, cols)[0])
        perm, _ = mx.column_perm(A, mx.COLPERM_FREQUENCY)
        assert np.array_equal(host(perm), oracle.colperm_frequency(ci, cols)[0])


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_csr5_and_ell_spmv(mx, cuda, handle, dtype):
    torch = cuda
    cases = [(n, rp, ci, v.astype(dtype), cols) for n, rp, ci, v, cols in larger_cases(mx)]
    for name in NAMES:
        g = gold(name)
        cases.append((name, g["rowPtr"], g["colIdx"], g["values"].astype(dtype), int(g["numCols"])))
    for name, rp, ci, v, cols in cases:
        A = device_csr(mx, rp, ci, v, cols)
        xh = mx.gen_vector(cols, 5, dtype=dtype)
        x = torch.from_numpy(xh).cuda()
        for sigma in (128, 256):
            m = mx.csr5_preprocess(A, sigma=sigma)
            for alpha, beta in ((1.0, 0.0), (2.0, -1.5)):
                y0 = mx.gen_vector(A.numRows, 6, dtype=dtype)
                y = torch.from_numpy(y0.copy()).cuda()
                mx.spmv_csr5(m, x, y, alpha, beta)
                torch.cuda.synchronize()
                check_y(y, y0, rp, ci, v, xh, alpha, beta)
            p = mx.Plan(handle, A, mx.make_variant(mx.KERNEL_CSR5, 256, 0, sigma // 32))
            y = torch.empty(A.numRows, dtype=x.dtype, device="cuda")
            p.exec(x, y)
            torch.cuda.synchronize()
            check_y(y, np.zeros(A.numRows, dtype), rp, ci, v, xh, 1.0, 0.0)
            p.destroy()
        lens = np.diff(rp)
        W = int(lens.max()) if len(lens) else 0
        e = mx.csr_to_ellpack(A)
        assert e.truncatedRows == 0 and e.numElements == W
        y0 = mx.gen_vector(A.numRows, 8, dtype=dtype)
        y = torch.from_numpy(y0.copy()).cuda()
        mx.spmv_ellpack(e, x, y, None, 0.5, 1.0)
        torch.cuda.synchronize()
        check_y(y, y0, rp, ci, v, xh, 0.5, 1.0)
        if A.numRows * W <= 2 * max(A.nnz, 1):
            p = mx.Plan(handle, A, mx.make_variant(mx.KERNEL_ELL))
            y = torch.empty(A.numRows, dtype=x.dtype, device="cuda")
            p.exec(x, y)
            torch.cuda.synchronize()
            check_y(y, np.zeros(A.numRows, dtype), rp, ci, v, xh, 1.0, 0.0)
            p.destroy()
        else:
            with pytest.raises(mx.SpmvError) as ex:
                mx.Plan(handle, A, mx.make_variant(mx.KERNEL_ELL))
            assert ex.value.status == -7


def test_csr5_deterministic(mx, cuda):
    torch = cuda
    name, rp, ci, v, cols = larger_cases(mx)[0]
    A = device_csr(mx, rp, ci, v, cols)
    m = mx.csr5_preprocess(A)
    x = torch.from_numpy(mx.gen_vector(cols, 9)).cuda()
    ys = []
    for _ in range(3):
        y = torch.empty(A.numRows, device="cuda")
        mx.spmv_csr5(m, x, y)
        ys.append(host(y))
    assert all(np.array_equal(ys[0], t) for t in ys[1:])
