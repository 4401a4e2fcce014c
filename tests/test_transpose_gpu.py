"""Transpose SpMV y = alpha*A^T*x + beta*y (the reference's declared
spmv_exec_transpose, spmv_api.h:70-78; its transpose kernel scatters with
float atomics, spmv_csr.cuh:105-107): the device transpose is bit-exact
against a numpy stable transpose, and y against the FP64 oracle run on
that transpose, bound 1e-5 (FP32) / 1e-13 (FP64) times sum |a x| per row."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu


def np_transpose(rp, ci, v, cols):
    rows = np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp))
    order = np.argsort(ci, kind="stable")
    trp = np.zeros(cols + 1, np.int64)
    np.add.at(trp, ci.astype(np.int64) + 1, 1)
    return np.cumsum(trp).astype(np.int32), rows[order].astype(np.int32), v[order]


def cases(mx):
    from muxi_spmv_gb300 import workloads as W
    out = {}
    s = W.scaled("powerlaw8m", 30000, seed=21)
    out["powerlaw"] = (*mx.generate(s), s.numCols)
    s = W.spec("poisson16k")
    out["poisson"] = (*mx.generate(s), s.numCols)
    rng = np.random.default_rng(4)
    lens = np.r_[np.zeros(20), rng.integers(0, 5, 700), np.zeros(9)].astype(np.int32)  # empty rows
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = np.concatenate([np.sort(rng.choice(2000, l, replace=False)) for l in lens]).astype(np.int32)
    out["rect_empty_cols"] = (rp, ci, rng.standard_normal(rp[-1]).astype(np.float32), 2000)
    out["no_nnz"] = (np.zeros(11, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 6)
    return out


@pytest.fixture(scope="module")
def mats(mx, cuda):
    return cases(mx)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_transpose_arrays_bit_exact(mx, cuda, mats, dtype):
    for name, (rp, ci, v, cols) in mats.items():
        A = device_csr(mx, rp, ci, v.astype(dtype), cols)
        B = mx.csr_transpose(A)
        cuda.cuda.synchronize()
        trp, tci, tv = np_transpose(rp, ci, v.astype(dtype), cols)
        assert np.array_equal(B.d_rowPtr.cpu().numpy(), trp), name
        assert np.array_equal(B.d_colIdx.cpu().numpy()[:len(tci)], tci), name
        assert np.array_equal(B.d_values.cpu().numpy()[:len(tv)], tv), name


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_transpose_spmv_matches_oracle(mx, cuda, mats, dtype):
    for name, (rp, ci, v, cols) in mats.items():
        rows = len(rp) - 1
        v = v.astype(dtype)
        A = device_csr(mx, rp, ci, v, cols)
        xh = mx.gen_vector(rows, 31, dtype=dtype)
        trp, tci, tv = np_transpose(rp, ci, v, cols)
        y_ref, absum = oracle.spmv_ref(trp, tci, tv, xh)
        for alpha, beta in ((1.0, 0.0), (-2.0, 0.5)):
            y0 = mx.gen_vector(cols, 8, dtype=dtype)
            y = cuda.from_numpy(y0.copy()).cuda() if cols else cuda.zeros(1, device="cuda")
            mx.spmv_csr_transpose(A, cuda.from_numpy(xh).cuda() if rows else cuda.zeros(1, device="cuda"), y,
                                  alpha, beta)
            cuda.cuda.synchronize()
            got = y.cpu().numpy()[:cols].astype(np.float64)
            want = alpha * y_ref + beta * y0.astype(np.float64)
            bound = tol_for(dtype) * (abs(alpha) * absum + abs(beta * y0.astype(np.float64)))
            assert (np.abs(got - want) <= bound + (0 if dtype == np.float64 else 1e-30)).all(), (name, alpha)


def test_transpose_is_deterministic(mx, cuda, mats):
    rp, ci, v, cols = mats["powerlaw"]
    A = device_csr(mx, rp, ci, v, cols)
    x = cuda.from_numpy(mx.gen_vector(len(rp) - 1, 3)).cuda()
    ys = []
    for _ in range(3):
        y = cuda.empty(cols, device="cuda")
        mx.spmv_csr_transpose(A, x, y)
        ys.append(y.cpu().numpy())
    assert all(np.array_equal(ys[0], b) for b in ys[1:])


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_plan_transpose_matches_oracle(mx, cuda, mats, dtype):
    """A plan answers both y = A x and y = A^T x; the transposed plan is built
    on the first transposed call and reused afterwards."""
    h = mx.spmv_create_handle()
    for name, (rp, ci, v, cols) in mats.items():
        rows = len(rp) - 1
        v = v.astype(dtype)
        A = device_csr(mx, rp, ci, v, cols)
        plan = mx.Plan(h, A)
        xh = mx.gen_vector(rows, 33, dtype=dtype)
        trp, tci, tv = np_transpose(rp, ci, v, cols)
        y_ref, absum = oracle.spmv_ref(trp, tci, tv, xh)
        x = cuda.from_numpy(xh).cuda() if rows else cuda.zeros(1, dtype=cuda.float32 if dtype == np.float32
                                                             else cuda.float64, device="cuda")
        for alpha, beta in ((1.0, 0.0), (-2.0, 0.5), (1.0, 0.0)):
            y0 = mx.gen_vector(cols, 9, dtype=dtype)
            y = cuda.from_numpy(y0.copy()).cuda() if cols else x.new_zeros(1)
            plan.exec(x, y, alpha, beta, transpose=True)
            cuda.cuda.synchronize()
            got = y.cpu().numpy()[:cols].astype(np.float64)
            want = alpha * y_ref + beta * y0.astype(np.float64)
            bound = tol_for(dtype) * (abs(alpha) * absum + abs(beta * y0.astype(np.float64)))
            assert (np.abs(got - want) <= bound + (0 if dtype == np.float64 else 1e-30)).all(), (name, alpha)
        # the plan still answers A x after the transposed calls
        xn = mx.gen_vector(cols, 34, dtype=dtype)
        yn_ref, absum_n = oracle.spmv_ref(rp, ci, v, xn)
        xd = cuda.from_numpy(xn).cuda() if cols else x.new_zeros(1)
        yd = x.new_zeros(max(rows, 1))
        plan.exec(xd, yd)
        cuda.cuda.synchronize()
        got = yd.cpu().numpy()[:rows].astype(np.float64)
        assert (np.abs(got - yn_ref) <= tol_for(dtype) * absum_n + (0 if dtype == np.float64 else 1e-30)).all(), name


def test_plan_refuses_conjugate(mx, cuda, mats):
    rp, ci, v, cols = mats["poisson"]
    A = device_csr(mx, rp, ci, v, cols)
    h = mx.spmv_create_handle()
    plan = mx.Plan(h, A)
    x = cuda.zeros(len(rp) - 1, device="cuda")
    y = cuda.zeros(cols, device="cuda")
    st = mx.lib().spmv_plan_exec_op_f32(h.raw, plan._p, 2, 1.0, x.data_ptr(), 0.0, y.data_ptr())  # SPMV_OP_CONJUGATE
    assert st == -7


@pytest.mark.parametrize("fmt", ["CSR", "CSR5", "ELL"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_convert_and_exec(mx, cuda, mats, fmt, dtype):
    """spmv_convert builds a plan in the named format; spmv_exec runs it for
    op = NORMAL and TRANSPOSE (the same bounds against the oracle)."""
    h = mx.spmv_create_handle()
    f = getattr(mx, "SPMV_FORMAT_" + fmt)
    for name, (rp, ci, v, cols) in mats.items():
        rows = len(rp) - 1
        if fmt == "ELL" and rows and np.diff(rp).max(initial=0) * rows > 2 * max(len(ci), 1):
            with pytest.raises(mx.SpmvError) as e:
                mx.Plan.from_format(h, device_csr(mx, rp, ci, v.astype(dtype), cols), f)
            assert e.value.status == -7, name
            continue
        v = v.astype(dtype)
        A = device_csr(mx, rp, ci, v, cols)
        plan = mx.Plan.from_format(h, A, f)
        if fmt == "CSR5":
            assert plan.variant.kernel == mx.KERNEL_CSR5
        if fmt == "ELL":
            assert plan.variant.kernel == mx.KERNEL_ELL
        zero = cuda.zeros(1, dtype=cuda.float32 if dtype == np.float32 else cuda.float64, device="cuda")
        for op, n_in, n_out, (prp, pci, pv) in ((mx.SPMV_OP_NORMAL, cols, rows, (rp, ci, v)),
                                                 (mx.SPMV_OP_TRANSPOSE, rows, cols, np_transpose(rp, ci, v, cols))):
            xh = mx.gen_vector(n_in, 35, dtype=dtype)
            y_ref, absum = oracle.spmv_ref(prp, pci, pv, xh)
            y0 = mx.gen_vector(n_out, 36, dtype=dtype)
            x = cuda.from_numpy(xh).cuda() if n_in else zero
            y = cuda.from_numpy(y0.copy()).cuda() if n_out else zero.clone()
            plan.exec_op(op, x, y, -1.5, 0.25)
            cuda.cuda.synchronize()
            got = y.cpu().numpy()[:n_out].astype(np.float64)
            want = -1.5 * y_ref + 0.25 * y0.astype(np.float64)
            bound = tol_for(dtype) * (1.5 * absum + abs(0.25 * y0.astype(np.float64)))
            assert (np.abs(got - want) <= bound + (0 if dtype == np.float64 else 1e-30)).all(), (name, fmt, op)


def test_convert_refuses_other_formats(mx, cuda, mats):
    rp, ci, v, cols = mats["poisson"]
    h = mx.spmv_create_handle()
    A = device_csr(mx, rp, ci, v, cols)
    for f in (mx.SPMV_FORMAT_COO, mx.SPMV_FORMAT_BSR, mx.SPMV_FORMAT_CSR2):
        with pytest.raises(mx.SpmvError) as e:
            mx.Plan.from_format(h, A, f)
        assert e.value.status == -7
