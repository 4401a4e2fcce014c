"""GPU parity of the CSR SpMV kernels against the FP64 CPU oracle, through
the C ABI.  Bound per row: |y - y_ref| <= tol * sum_j |a_ij x_j| with
tol = 1e-5 (FP32) and 1e-13 (FP64)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def build_cases(mx):
    from muxi_spmv_gb300 import workloads as W
    cases = {}
    cases["poisson16k"] = (*mx.generate(W.spec("poisson16k")), 16384)
    s = W.scaled("powerlaw8m", 60000, seed=2)
    cases["powerlaw60k"] = (*mx.generate(s), s.numCols)
    s = W.scaled("stencil2d_4096", 100 * 100, seed=3)
    cases["stencil2d"] = (*mx.generate(s), s.numCols)
    s = W.scaled("stencil3d_256", 20 ** 3, seed=4)
    cases["stencil3d"] = (*mx.generate(s), s.numCols)
    # One 65,536-nnz row among short ones (the longest row the power-law law allows).
    rng = np.random.default_rng(5)
    lens = np.r_[rng.integers(0, 4, 300), 65536, rng.integers(0, 4, 300)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    cols = 70000
    ci = np.sort(rng.integers(0, cols, rp[-1]).astype(np.int32))
    v = rng.standard_normal(rp[-1]).astype(np.float32)
    cases["longrow"] = (rp, ci, v, cols)
    # Empty rows everywhere, including leading and trailing runs.
    lens = np.r_[np.zeros(50), rng.integers(0, 3, 2000) * (rng.random(2000) < 0.4), np.zeros(70)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = rng.integers(0, 500, rp[-1]).astype(np.int32)
    v = rng.standard_normal(rp[-1]).astype(np.float32)
    cases["empties"] = (rp, ci, v, 500)
    # Leading empty rows before a row longer than two tiles of every size: the
    # first tile lies inside one row and must still write the empty rows.
    lens = np.r_[np.zeros(7), 3000, rng.integers(0, 5, 40), np.zeros(5)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = np.sort(rng.integers(0, 4000, rp[-1]).astype(np.int32))
    cases["lead_empty_longrow"] = (rp, ci, rng.standard_normal(rp[-1]).astype(np.float32), 4000)
    cases["one_row"] = (np.array([0, 5], np.int32), np.array([0, 1, 1, 7, 9], np.int32),
                        np.array([1, 2, 3, 4, 5], np.float32), 10)
    cases["no_nnz"] = (np.zeros(33, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 33)
    return cases


@pytest.fixture(scope="module")
def cases(mx):
    return build_cases(mx)


VARIANTS = [("mvec", 3, 256, 8, 0, 4), ("mvec", 3, 256, 4, 0, 4), ("mvec", 3, 256, 16, 0, 4),
            ("mvec", 3, 128, 12, 0, 4), ("mvec", 3, 128, 8, 0, 4),
            ("merge", 3, 256, 7, 0, 1), ("merge", 3, 256, 3, 0, 1), ("merge", 3, 256, 11, 0, 1),
            ("merge", 3, 128, 5, 0, 1), ("merge", 3, 128, 9, 0, 1),
            ("scalar", 1, 256, 0, 1, 1), ("vec2", 2, 256, 0, 2, 1), ("vec4q", 2, 128, 0, 4, 4),
            ("vec8", 2, 512, 0, 8, 1), ("vec8q", 2, 256, 0, 8, 4), ("vec16q", 2, 256, 0, 16, 4),
            ("vec32", 2, 256, 0, 32, 1), ("vec32q", 2, 256, 0, 32, 4), ("vec1q", 2, 256, 0, 1, 4),
            ("vec4", 2, 64, 0, 4, 1), ("vec2q", 2, 1024, 0, 2, 4), ("scalar", 1, 1024, 0, 1, 1)]


def run_variant(mx, cuda, A, x, y, var, alpha, beta):
    name, kernel, block, ipt, tpr, vw = var
    v = mx.make_variant(kernel, block, tpr, ipt, vw)
    mx.spmv_csr_variant(v, A, x, y, alpha, beta)
    cuda.cuda.synchronize()


def check(y_dev, y0, A, x_host, alpha, beta):
    y = y_dev.cpu().numpy()
    yr, a = oracle.spmv_ref(A.rowPtr, A.colIdx, A.values, x_host)
    want = alpha * yr + (beta * y0.astype(np.float64) if beta != 0 else 0.0)
    scale = abs(alpha) * a + (abs(beta) * np.abs(y0.astype(np.float64)) if beta != 0 else 0.0)
    tol = tol_for(A.dtype)
    err = np.abs(y.astype(np.float64) - want)
    # y = A x is held to the bound itself; with alpha != 1 or beta != 0 the
    # epilogue adds one rounding of alpha*s + beta*y in the value type
    eps = np.finfo(A.dtype).eps
    bound = tol * scale + (2 * eps * np.abs(want) if (alpha != 1.0 or beta != 0.0) else 0.0)
    bad = np.flatnonzero(err > bound)
    assert bad.size == 0, f"{bad.size} rows out of bound, first {bad[:5]}, err {err[bad[:5]]}, bound {bound[bad[:5]]}"


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("var", VARIANTS, ids=[v[0] + str(v[3] or "") + "b" + str(v[2]) for v in VARIANTS])
def test_variants_match_oracle(mx, cuda, cases, var, dtype):
    torch = cuda
    for name, (rp, ci, v, cols) in cases.items():
        A = device_csr(mx, rp, ci, v.astype(dtype), cols)
        xh = mx.gen_vector(cols, 77, dtype=dtype)
        x = torch.from_numpy(xh).cuda()
        for alpha, beta in ((1.0, 0.0), (-0.5, 2.0)):
            y0 = mx.gen_vector(A.numRows, 99, dtype=dtype)
            y = torch.from_numpy(y0.copy()).cuda()
            run_variant(mx, torch, A, x, y, var, alpha, beta)
            check(y, y0, A, xh, alpha, beta)


# BAND: (block, ept, window in 1,024-element units, tiles per warp); the
# 1K and 2K windows leave most gathers of the larger cases outside the window.
PLAN_VARIANTS = [("band", 7, 512, 16, 0, 0), ("band", 7, 512, 8, 0, 0), ("band", 7, 1024, 16, 0, 2),
                 ("band", 7, 256, 8, 1, 1), ("band", 7, 256, 16, 2, 3), ("band", 7, 1024, 8, 4, 16),
                 ("band", 7, 1024, 8, 16, 25), ("band", 7, 1024, 8, 0, 0),
                 ("csr5_512", 4, 256, 16, 4, 0), ("csr5_128", 4, 256, 4, 4, 0),
                 ("csr5o_128", 4, 256, 4, 32, 0), ("csr5o_256", 4, 256, 8, 32, 0), ("csr5o_512", 4, 256, 16, 32, 0),
                 ("csr5o_b128", 4, 128, 8, 32, 0), ("csr5o_b512", 4, 512, 8, 32, 0), ("csr5o_b1024", 4, 1024, 8, 32, 0),
                 ("csr5r_256c3", 4, 256, 8, 32, 3), ("csr5r_512c64", 4, 512, 4, 32, 64),
                 ("csr5r_1024c8", 4, 1024, 8, 32, 8), ("csr5r_1024c1", 4, 1024, 16, 32, 1),
                 ("csr5r_640sm", 4, 640, 16, 32, 1 << 20), ("csr5r_384c2", 4, 384, 8, 32, 2),
                 ("csr5pf_1024sm", 4, 1024, 8, 64, 1 << 20), ("csr5pf_512c3", 4, 512, 16, 64, 3),
                 ("stream", 8, 512, 0, 0, 0), ("stream", 8, 1024, 8, 0, 3), ("stream", 8, 1024, 8, 0, 2),
                 ("stream", 8, 768, 16, 0, 2)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("var", PLAN_VARIANTS, ids=[f"{v[0]}b{v[2]}e{v[3]}w{v[4]}" for v in PLAN_VARIANTS])
def test_plan_variants_match_oracle(mx, cuda, handle, cases, var, dtype):
    """Plan-only kernels (tile metadata built at plan creation): the x-window
    kernel (large and small windows), CSR5 at every tile size and block shape,
    CSR5 block ranges (plain, one per SM, prefetching) and the bulk-copy-fed
    stream kernel, on every edge case."""
    torch = cuda
    name_, kernel, block, ept, vw, tpr = var
    if kernel == mx.KERNEL_STREAM and dtype == np.float64 and not (ept in (0, 8) and block in (512, 1024)):
        pytest.skip("FP64 stream shapes: 8 nonzeros per lane at 512 (3 stages) or 1024 threads (2 stages)")
    if kernel == mx.KERNEL_STREAM and dtype == np.float64 and block == 1024:
        tpr = 2
    for name, (rp, ci, v, cols) in cases.items():
        A = device_csr(mx, rp, ci, v.astype(dtype), cols)
        xh = mx.gen_vector(cols, 77, dtype=dtype)
        x = torch.from_numpy(xh).cuda()
        p = mx.Plan(handle, A, mx.make_variant(kernel, block, tpr, ept, vw))
        for alpha, beta in ((1.0, 0.0), (-0.5, 2.0)):
            y0 = mx.gen_vector(A.numRows, 99, dtype=dtype)
            y = torch.from_numpy(y0.copy()).cuda()
            p.exec(x, y, alpha, beta)
            torch.cuda.synchronize()
            assert p.device_error() == 0
            check(y, y0, A, xh, alpha, beta)
        p.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_band_unaligned_x_reads_global(mx, cuda, handle, cases, dtype):
    """x one element past a 16-byte boundary: the window cannot be bulk-copied,
    so the x-window kernel gathers every column from global memory."""
    torch = cuda
    rp, ci, v, cols = cases["powerlaw60k"]
    A = device_csr(mx, rp, ci, v.astype(dtype), cols)
    xh = mx.gen_vector(cols, 77, dtype=dtype)
    xbuf = torch.zeros(cols + 4, dtype=torch.float32 if dtype == np.float32 else torch.float64, device="cuda")
    x = xbuf[1:cols + 1]
    x.copy_(torch.from_numpy(xh))
    assert x.data_ptr() % 16 != 0
    p = mx.Plan(handle, A, mx.make_variant(mx.KERNEL_BAND, 512, 0, 8, 0))
    y = torch.empty(A.numRows, dtype=x.dtype, device="cuda")
    p.exec(x, y)
    torch.cuda.synchronize()
    assert p.device_error() == 0
    check(y, np.zeros(A.numRows, dtype), A, xh, 1.0, 0.0)
    p.destroy()


@pytest.mark.parametrize("kind", ["band", "band1024", "stream"])
def test_bulk_copy_wait_runs_out_and_reports(mx, cuda, handle, cases, kind):
    """Waits on bulk copies are bounded.  With one arrival of each copy
    barrier held back, the waits run out after 100,000 clocks; the kernel
    makes the arrivals itself so its copies land, returns, and the plan
    reports code 2 (BAND window) or 3 (STREAM tile slots) as SpmvError.  The
    context stays usable: the next normal execution of the same plan matches
    the oracle.  band1024 is the window kernel's shape the selector offers
    (one 1,024-thread CTA per SM, next tile prefetched, 16-byte tile loads)."""
    torch = cuda
    rp, ci, v, cols = cases["powerlaw60k"]
    A = device_csr(mx, rp, ci, v, cols)
    xh = mx.gen_vector(cols, 77)
    x = torch.from_numpy(xh).cuda()
    var = {"band": mx.make_variant(mx.KERNEL_BAND, 512, 0, 16, 0),
           "band1024": mx.make_variant(mx.KERNEL_BAND, 1024, 25, 8, 14),
           "stream": mx.make_variant(mx.KERNEL_STREAM, 512, 3, 16, 0)}[kind]
    p = mx.Plan(handle, A, var)
    y = torch.zeros(A.numRows, device="cuda")
    p.inject_wait_timeout(True)
    p.exec(x, y)
    torch.cuda.synchronize()
    with pytest.raises(mx.SpmvError, match="code 3" if kind == "stream" else "code 2"):
        p.device_error()
    assert p.device_error() == 0  # reading the word cleared it
    p.inject_wait_timeout(False)
    p.exec(x, y)
    torch.cuda.synchronize()
    assert p.device_error() == 0
    check(y, np.zeros(A.numRows, np.float32), A, xh, 1.0, 0.0)
    p.destroy()
    q = mx.Plan(handle, A, mx.make_variant(mx.KERNEL_CSR5, 128, 0, 16, 32))  # no bounded wait to inject into
    with pytest.raises(mx.SpmvError):
        q.inject_wait_timeout(True)
    q.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_stateless_and_merge_based(mx, cuda, cases, dtype):
    torch = cuda
    for name, (rp, ci, v, cols) in cases.items():
        A = device_csr(mx, rp, ci, v.astype(dtype), cols)
        xh = mx.gen_vector(cols, 7, dtype=dtype)
        x = torch.from_numpy(xh).cuda()
        y = torch.full((max(A.numRows, 1),), float("nan"), dtype=x.dtype, device="cuda")[: A.numRows]
        mx.spmv_csr(A, x, y)  # beta = 0 never reads y: NaN must not leak
        torch.cuda.synchronize()
        check(y, np.zeros(A.numRows, dtype), A, xh, 1.0, 0.0)
        y2 = torch.full_like(y, float("nan"))
        mx.spmv_merge_based(A, x, y2)
        torch.cuda.synchronize()
        check(y2, np.zeros(A.numRows, dtype), A, xh, 1.0, 0.0)


def test_merge_is_deterministic(mx, cuda, cases):
    torch = cuda
    rp, ci, v, cols = cases["powerlaw60k"]
    A = device_csr(mx, rp, ci, v, cols)
    x = torch.from_numpy(mx.gen_vector(cols, 1)).cuda()
    ys = []
    for _ in range(3):
        y = torch.empty(A.numRows, device="cuda")
        mx.spmv_csr(A, x, y)
        ys.append(y.cpu().numpy())
    assert all(np.array_equal(ys[0], t) for t in ys[1:])


def test_kat_diagonal(mx, cuda):
    """tests/correctness/test_spmv.cu:44-115 through the C ABI."""
    torch = cuda
    g = np.load(GOLD / "kat_diagonal.npz")
    A = device_csr(mx, g["rowPtr"], g["colIdx"], g["values"], len(g["x"]))
    h = mx.spmv_create_handle()
    assert h.warpSize == 32 and h.smCount > 0
    x = torch.from_numpy(g["x"]).cuda()
    y = torch.zeros_like(x)
    o = mx.spmv_default_opts(sync=True)
    mx.spmv_csr(A, x, y, 1.0, 0.0, o)
    assert np.max(np.abs(y.cpu().numpy() - g["y_expected"])) <= 1e-5
    h.destroy()


@pytest.mark.parametrize("name", ["poisson_2k", "powerlaw_3k", "stencil2d_40", "empty_rows"])
def test_golden_index_outputs(mx, cuda, name):
    """Merge partitions and path coordinates from the GPU equal the
    reference's (golden fixtures from the reference's own code)."""
    torch = cuda
    g = dict(np.load(GOLD / f"{name}.npz"))
    A = device_csr(mx, g["rowPtr"], g["colIdx"], g["values"], int(g["numCols"]))
    P = int(g["merge_P"])
    assert mx.merge_default_partitions(A.numRows, A.nnz) == P
    pos = mx.compute_merge_partitions(A.numRows, A.nnz, P)
    assert np.array_equal(pos.cpu().numpy(), g["merge_pos"])
    r, z = mx.merge_path_search(A, torch.from_numpy(g["merge_diag"]).cuda())
    assert np.array_equal(r.cpu().numpy(), g["merge_row"]) and np.array_equal(z.cpu().numpy(), g["merge_nnz"])
    # SpMV on the fixture matches the FP64 oracle and bounds the reference loop
    x = torch.from_numpy(g["x"]).cuda()
    y = torch.empty(A.numRows, device="cuda")
    mx.spmv_csr(A, x, y)
    torch.cuda.synchronize()
    check(y, np.zeros(A.numRows, np.float32), A, g["x"], 1.0, 0.0)


def test_merge_search_all_diagonals(mx, cuda, cases):
    torch = cuda
    for name in ("empties", "longrow", "one_row", "no_nnz"):
        rp, ci, v, cols = cases[name]
        A = device_csr(mx, rp, ci, v, cols)
        diag = np.arange(A.numRows + A.nnz + 1, dtype=np.int32)
        r, z = mx.merge_path_search(A, torch.from_numpy(diag).cuda())
        r2, z2 = oracle.merge_search(rp, A.nnz, diag)
        assert np.array_equal(r.cpu().numpy(), r2) and np.array_equal(z.cpu().numpy(), z2)
        for P in (1, 3, mx.merge_default_partitions(A.numRows, A.nnz)):
            pos = mx.compute_merge_partitions(A.numRows, A.nnz, P)
            assert np.array_equal(pos.cpu().numpy(), oracle.merge_partitions(A.numRows, A.nnz, P))


def test_plans(mx, cuda, handle, cases):
    torch = cuda
    rp, ci, v, cols = cases["powerlaw60k"]
    for dtype in (np.float32, np.float64):
        A = device_csr(mx, rp, ci, v.astype(dtype), cols)
        xh = mx.gen_vector(cols, 3, dtype=dtype)
        x = torch.from_numpy(xh).cuda()
        for var in (None, mx.make_variant(mx.KERNEL_HEURISTIC), mx.make_variant(mx.KERNEL_MERGE, 128, 0, 9),
                    mx.make_variant(mx.KERNEL_VECTOR, 256, 8, 0, 4)):
            p = mx.Plan(handle, A, var)
            y0 = mx.gen_vector(A.numRows, 4, dtype=dtype)
            y = torch.from_numpy(y0.copy()).cuda()
            p.exec(x, y, 1.5, -1.0)
            torch.cuda.synchronize()
            check(y, y0, A, xh, 1.5, -1.0)
            p.destroy()
    # heuristic resolves to the reference's rule (avgNnz < 32 -> scalar)
    A = device_csr(mx, rp, ci, v, cols)
    p = mx.Plan(handle, A, mx.make_variant(mx.KERNEL_HEURISTIC))
    assert p.variant.kernel == mx.KERNEL_SCALAR
    p.destroy()


def test_f64_auto_takes_block_ranges_on_large_near_diagonal_matrices(mx, cuda, handle, cases):
    """FP64 AUTO plans (no model) take one range of tiles per resident block
    when every warp of those ranges gets at least 8 tiles and most sampled
    nonzeros lie within 4,096 columns of the diagonal; otherwise the FP64
    default (one 256-nonzero tile per warp, 128-thread blocks).  The ranges'
    result matches the oracle at the FP64 bound."""
    torch = cuda
    from muxi_spmv_gb300 import workloads as W
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    need = sms * 32 * 8 * 256  # nonzeros that give every warp 8 tiles of 256
    R = mx.RANGE_PER_RESIDENT_BLOCK

    def auto_variant(rp, ci, v, cols):
        A = device_csr(mx, rp, ci, v.astype(np.float64), cols)
        p = mx.Plan(handle, A)
        pv = p.variant
        return A, p, (pv.kernel, pv.blockSize, pv.threadsPerRow, pv.itemsPerThread, pv.vectorWidth)

    # near-diagonal and large: a 2D 5-point grid of about need/5 * 1.2 rows
    spec = W.scaled("stencil2d_4096", int(need / 5 * 1.2), seed=7)
    rp, ci, v = mx.generate(spec)
    assert rp[-1] >= need
    A, p, key = auto_variant(rp, ci, v, spec.numCols)
    assert key == (mx.KERNEL_CSR5, 1024, R, 8, 32)
    xh = mx.gen_vector(spec.numCols, 5, dtype=np.float64)
    y = torch.zeros(A.numRows, dtype=torch.float64, device="cuda")
    p.exec(torch.from_numpy(xh).cuda(), y)
    torch.cuda.synchronize()
    check(y, np.zeros(A.numRows), A, xh, 1.0, 0.0)
    p.destroy()
    del A
    # large but uniform columns: the default
    spec = W.scaled("poisson16k", int(need / 12 * 1.2), seed=8)
    rp, ci, v = mx.generate(spec)
    assert rp[-1] >= need
    A, p, key = auto_variant(rp, ci, v, spec.numCols)
    assert key == (mx.KERNEL_CSR5, 128, 0, 8, 32)
    p.destroy()
    del A
    # small: the default
    rp, ci, v, cols = cases["powerlaw60k"]
    A, p, key = auto_variant(rp, ci, v, cols)
    assert key == (mx.KERNEL_CSR5, 128, 0, 8, 32)
    p.destroy()


def test_f64_interior_tiles_over_wide_exponent_ranges(mx, cuda, handle):
    """FP64 tiles inside one row sum their lanes in 64-bit fixed point below
    the largest lane's exponent: long rows whose products span 1e-300 to
    1e300, cancel to a small remainder, sit near the top of the range, or are
    tiny enough to take the FP64 fallback, each within the FP64 bound; a row
    of integer products comes out exact."""
    torch = cuda
    rng = np.random.default_rng(57)
    cols = 60_000
    lens = [40_000, 20_000, 12_000, 12_000, 9_000] + [int(z) for z in rng.integers(1, 40, 500)]
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = np.concatenate([np.sort(rng.choice(cols, l, replace=False)) for l in lens]).astype(np.int32)
    v = rng.standard_normal(rp[-1])
    s0, s1, s2, s3, s4 = (slice(rp[i], rp[i + 1]) for i in range(5))
    v[s0] *= 10.0 ** rng.uniform(-300, 300, lens[0])  # products over 600 decades
    v[s1] = np.where(np.arange(lens[1]) % 2 == 0, 1e16, -1e16) * (1 + 1e-12 * rng.standard_normal(lens[1]))
    v[s2] *= 1e-305                                   # tiny: largest exponent below the fixed-point range
    v[s3] *= 1e300                                    # near the top of the range
    v[s4] = rng.integers(-1000, 1001, lens[4]).astype(np.float64)
    xh = rng.uniform(-1, 1, cols)
    xh[ci[s4]] = rng.integers(-3, 4, lens[4]).astype(np.float64)  # row 4: integer products
    A = device_csr(mx, rp, ci, v, cols)
    x = torch.from_numpy(xh).cuda()
    exact4 = int(np.sum(v[s4].astype(np.int64) * xh[ci[s4]].astype(np.int64)))
    R = mx.RANGE_PER_RESIDENT_BLOCK
    for var in (None, mx.make_variant(mx.KERNEL_CSR5, 128, 0, 16, 32), mx.make_variant(mx.KERNEL_CSR5, 128, 0, 8, 32),
                mx.make_variant(mx.KERNEL_CSR5, 1024, R, 8, mx.CSR5_ORDERED_PREFETCH)):
        p = mx.Plan(handle, A, var)
        y = torch.zeros(A.numRows, dtype=torch.float64, device="cuda")
        p.exec(x, y)
        torch.cuda.synchronize()
        check(y, np.zeros(A.numRows), A, xh, 1.0, 0.0)
        assert y[4].item() == float(exact4)
        p.destroy()


def test_unused_nonfinite_x_does_not_leak(mx, cuda, handle):
    """Padding slots and masked lanes read x[0] or other columns without using
    them: an Inf / NaN in columns no nonzero references must not reach y."""
    torch = cuda
    rng = np.random.default_rng(31)
    lens = np.r_[rng.integers(1, 9, 3000), 700, rng.integers(1, 6, 2000)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    cols = 6000
    ci = np.concatenate([np.sort(rng.choice(np.arange(2, cols), l, replace=False)) for l in lens]).astype(np.int32)
    v = rng.standard_normal(rp[-1]).astype(np.float32)
    assert rp[-1] % 512 != 0  # a partial last tile
    A = device_csr(mx, rp, ci, v, cols)
    xh = mx.gen_vector(cols, 3)
    xh[0], xh[1] = np.inf, np.nan  # columns 0 and 1 are never referenced
    x = torch.from_numpy(xh).cuda()
    y_ref, _ = oracle.spmv_ref(rp, ci, v, xh)
    assert np.isfinite(y_ref).all()
    variants = [None, mx.make_variant(mx.KERNEL_CSR5, 128, 0, 4, 32), mx.make_variant(mx.KERNEL_CSR5, 256, 0, 8, 1),
                mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4), mx.make_variant(mx.KERNEL_MERGE, 128, 0, 9),
                mx.make_variant(mx.KERNEL_VECTOR, 256, 8, 0, 4), mx.make_variant(mx.KERNEL_SCALAR, 128),
                mx.make_variant(mx.KERNEL_ELL), mx.make_variant(mx.KERNEL_BAND, 256, 0, 8)]
    for var in variants:
        try:
            p = mx.Plan(handle, A, var)
        except mx.SpmvError:
            continue  # a shape this matrix does not take (ELL padding gate)
        y = torch.zeros(A.numRows, device="cuda")
        p.exec(x, y)
        torch.cuda.synchronize()
        assert torch.isfinite(y).all(), var.as_dict() if var is not None else "auto"
        p.destroy()
    y = torch.zeros(A.numRows, device="cuda")
    mx.spmv_csr(A, x, y)
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()


def test_plan_copy_owns_the_matrix(mx, cuda, handle, cases):
    """SPMV_PLAN_COPY: the plan runs from its own copy after the caller's
    arrays are overwritten (the default borrows them)."""
    torch = cuda
    rp, ci, v, cols = cases["powerlaw60k"]
    A = device_csr(mx, rp, ci, v, cols)
    xh = mx.gen_vector(cols, 8)
    x = torch.from_numpy(xh).cuda()
    for var in (None, mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4), mx.make_variant(mx.KERNEL_VECTOR, 256, 4, 0, 4)):
        p = mx.Plan(handle, A, var, copy=True)
        A.d_colIdx.fill_(0)
        A.d_values.fill_(float("nan"))
        A.d_rowPtr.fill_(0)
        y = torch.zeros(A.numRows, device="cuda")
        p.exec(x, y)
        torch.cuda.synchronize()
        A.copyToDevice()
        check(y, np.zeros(A.numRows, np.float32), A, xh, 1.0, 0.0)
        p.destroy()


def test_plan_exec_replays_from_a_cuda_graph(mx, cuda, cases):
    """A plan allocates nothing at execution and its fix-up launch (with the
    programmatic-dependent-launch attribute) captures: ten SpMVs recorded into
    one CUDA graph replay with the same bits as direct executions."""
    torch = cuda
    for name in ("powerlaw60k", "empties", "lead_empty_longrow"):
        rp, ci, v, cols = cases[name]
        A = device_csr(mx, rp, ci, v, cols)
        xh = mx.gen_vector(cols, 12)
        x = torch.from_numpy(xh).cuda()
        s = torch.cuda.Stream()
        h = mx.spmv_create_handle()
        h.set_stream(s)
        for var in (None, mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4), mx.make_variant(mx.KERNEL_ELL)):
            try:
                p = mx.Plan(h, A, var)
            except mx.SpmvError:
                continue  # ELL refused (padding above 2x)
            y_direct = torch.zeros(A.numRows, device="cuda")
            with torch.cuda.stream(s):
                p.exec(x, y_direct)
            s.synchronize()
            y = torch.zeros(A.numRows, device="cuda")
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                for _ in range(10):
                    p.exec(x, y)
            y.zero_()
            g.replay()
            torch.cuda.synchronize()
            assert torch.equal(y, y_direct), (name, var.as_dict() if var is not None else "auto")
            p.destroy()
        h.destroy()


def test_stats(mx, cuda, cases):
    for name in ("powerlaw60k", "empties", "no_nnz"):
        rp, ci, v, cols = cases[name]
        A = device_csr(mx, rp, ci, v, cols)
        assert mx.count_distinct_columns(A) == oracle.distinct_columns(ci, cols)
        assert mx.validate_csr(A) == 0
    rp, ci, v, cols = cases["powerlaw60k"]
    bad = ci.copy()
    bad[[3, 10, 99]] = cols + 5
    A = device_csr(mx, rp, bad, v, cols)
    assert mx.validate_csr(A) == 3


def test_errors_on_device(mx, cuda, handle, cases):
    rp, ci, v, cols = cases["poisson16k"]
    A = device_csr(mx, rp, ci, v, cols)
    with pytest.raises(mx.SpmvError) as e:
        mx.spmv_csr_variant(mx.make_variant(mx.KERNEL_MERGE, 256, 0, 6), A, A.d_values, A.d_values)
    assert e.value.status == -9
    with pytest.raises(mx.SpmvError) as e:
        mx.Plan(handle, A, mx.make_variant(mx.KERNEL_VECTOR, 256, 3))
    assert e.value.status == -9
