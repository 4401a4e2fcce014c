"""Host-to-host pipeline (the pinned-memory / multi-stream path of the
reference's tests/test_pinned_memory.cu:245-380): every request's y, copied
back slice by slice while later slices and requests run, is checked row by
row against the FP64 oracle (bound 1e-5 FP32 / 1e-13 FP64 times sum |a x|,
plus |beta*y0| when beta != 0).  Also: kernels that read 16-byte quads on
colIdx / values that are not 16-byte aligned (offset views) run a fallback
with the same results."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu


def cases(mx):
    from muxi_spmv_gb300 import workloads as W
    out = {}
    s = W.scaled("powerlaw8m", 40000, seed=5)
    out["powerlaw"] = (*mx.generate(s), s.numCols)
    rng = np.random.default_rng(11)
    lens = np.r_[np.zeros(13), rng.integers(0, 9, 3000), [20000], np.zeros(40), rng.integers(1, 4, 500),
                 np.zeros(7)].astype(np.int32)  # empty runs and one long row
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = np.concatenate([np.sort(rng.choice(25000, l, replace=False)) for l in lens]).astype(np.int32)
    out["ragged"] = (rp, ci, rng.standard_normal(rp[-1]).astype(np.float32), 25000)
    out["one_row"] = (np.array([0, 5000], np.int32), np.arange(5000, dtype=np.int32),
                      rng.standard_normal(5000).astype(np.float32), 5000)
    out["no_nnz"] = (np.zeros(9, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 4)
    return out


@pytest.fixture(scope="module")
def mats(mx, cuda):
    return cases(mx)


def check_rows(got, y_ref, absum, alpha, beta, y0, dtype, what):
    want = alpha * y_ref + beta * y0.astype(np.float64)
    bound = tol_for(dtype) * (abs(alpha) * absum + abs(beta * y0.astype(np.float64)))
    bad = np.abs(got.astype(np.float64) - want) > bound + (0 if dtype == np.float64 else 1e-30)
    assert not bad.any(), (what, int(bad.sum()), np.flatnonzero(bad)[:5])


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("slices,depth", [(1, 1), (3, 2), (8, 2), (64, 3)])
def test_pipeline_matches_oracle(mx, cuda, mats, dtype, slices, depth):
    h = mx.spmv_create_handle()
    for name, (rp, ci, v, cols) in mats.items():
        rows = len(rp) - 1
        v = v.astype(dtype)
        A = device_csr(mx, rp, ci, v, cols)
        pipe = mx.Pipeline(h, A, slices=slices, depth=depth)
        info = pipe.info()
        assert 1 <= info["slices"] <= slices and info["depth"] == depth, (name, info)
        # five requests with distinct x, alternating alpha / beta
        reqs = []
        for i in range(5):
            xh = cuda.from_numpy(mx.gen_vector(max(cols, 1), 100 + i, dtype=dtype)).pin_memory()
            y0 = mx.gen_vector(max(rows, 1), 200 + i, dtype=dtype)
            yh = cuda.from_numpy(y0.copy()).pin_memory()
            alpha, beta = (1.0, 0.0) if i % 2 == 0 else (-1.5, 0.25)
            pipe.submit(xh, yh, alpha, beta)
            reqs.append((xh, yh, y0, alpha, beta))
        pipe.wait()
        for i, (xh, yh, y0, alpha, beta) in enumerate(reqs):
            y_ref, absum = oracle.spmv_ref(rp, ci, v, xh.numpy()[:cols])
            check_rows(yh.numpy()[:rows], y_ref, absum, alpha, beta, y0[:rows], dtype, (name, i))
        pipe.destroy()


def test_pipeline_slices_keep_aligned_starts(mx, cuda, mats):
    """Slice boundaries move to rows whose first nonzero is a multiple of 4,
    so a merge-path variant reading 16-byte quads keeps them on every slice."""
    rp, ci, v, cols = mats["powerlaw"]
    h = mx.spmv_create_handle()
    A = device_csr(mx, rp, ci, v, cols)
    var = mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4)
    pipe = mx.Pipeline(h, A, var, slices=16, depth=2)
    info = pipe.info()
    assert info["variant"]["kernel"] == mx.KERNEL_MERGE and info["variant"]["vectorWidth"] == 4
    xh = cuda.from_numpy(mx.gen_vector(cols, 7)).pin_memory()
    yh = cuda.empty(len(rp) - 1).pin_memory()
    pipe.submit(xh, yh)
    pipe.wait()
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh.numpy())
    check_rows(yh.numpy(), y_ref, absum, 1.0, 0.0, np.zeros(len(rp) - 1, np.float32), np.float32, "merge-vec slices")


def test_pipeline_order_and_join_with_a_stream(mx, cuda, mats):
    rp, ci, v, cols = mats["powerlaw"]
    h = mx.spmv_create_handle()
    A = device_csr(mx, rp, ci, v, cols)
    pipe = mx.Pipeline(h, A)
    s = cuda.cuda.Stream()
    xh = cuda.from_numpy(mx.gen_vector(cols, 9)).pin_memory()
    yh = cuda.zeros(len(rp) - 1).pin_memory()
    e0, e1 = cuda.cuda.Event(enable_timing=True), cuda.cuda.Event(enable_timing=True)
    e0.record(s)
    pipe.order_after(s)
    pipe.submit(xh, yh)
    pipe.join(s)
    e1.record(s)
    e1.synchronize()
    assert e0.elapsed_time(e1) > 0
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh.numpy())
    check_rows(yh.numpy(), y_ref, absum, 1.0, 0.0, np.zeros(len(rp) - 1, np.float32), np.float32, "joined")
    pipe.wait()


def offset_csr(mx, cuda, rp, ci, v, cols):
    """A device CSR whose colIdx / values start one element past a 16-byte
    boundary (views into larger buffers)."""
    A = mx.CSRMatrix(rp, ci, v, cols)
    tdt = cuda.float32 if v.dtype == np.float32 else cuda.float64
    A.d_rowPtr = cuda.from_numpy(rp).cuda()
    cbuf = cuda.zeros(len(ci) + 4, dtype=cuda.int32, device="cuda")
    vbuf = cuda.zeros(len(v) + 4, dtype=tdt, device="cuda")
    cbuf[1:1 + len(ci)] = cuda.from_numpy(ci).cuda()
    vbuf[1:1 + len(v)] = cuda.from_numpy(v).cuda()
    A.d_colIdx, A.d_values = cbuf[1:1 + len(ci)], vbuf[1:1 + len(v)]
    A._bufs = (cbuf, vbuf)
    assert A.d_colIdx.data_ptr() % 16 != 0 and A.d_values.data_ptr() % 16 != 0
    return A


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_unaligned_arrays_take_the_fallback(mx, cuda, mats, dtype):
    rp, ci, v, cols = mats["ragged"]
    v = v.astype(dtype)
    A = offset_csr(mx, cuda, rp, ci, v, cols)
    xh = mx.gen_vector(cols, 3, dtype=dtype)
    x = cuda.from_numpy(xh).cuda()
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    rows = len(rp) - 1
    zero = np.zeros(rows, dtype)
    h = mx.spmv_create_handle()
    # stateless default (merge-path with 16-byte quads when aligned)
    y = cuda.zeros(rows, dtype=x.dtype, device="cuda")
    mx.spmv_csr(A, x, y)
    cuda.cuda.synchronize()
    check_rows(y.cpu().numpy(), y_ref, absum, 1.0, 0.0, zero, dtype, "stateless")
    # plans: merge quads -> per-item consumer; lane-contiguous CSR5 -> ordered tiles
    for var in (mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4), mx.make_variant(mx.KERNEL_CSR5, 256, 0, 8, 1),
                mx.make_variant(mx.KERNEL_VECTOR, 256, 4, 0, 4)):
        plan = mx.Plan(h, A, var)
        if var.kernel == mx.KERNEL_MERGE:
            assert plan.variant.as_dict()["vectorWidth"] == 1
        y = cuda.zeros(rows, dtype=x.dtype, device="cuda")
        plan.exec(x, y)
        cuda.cuda.synchronize()
        check_rows(y.cpu().numpy(), y_ref, absum, 1.0, 0.0, zero, dtype, var.as_dict())
        plan.destroy()
