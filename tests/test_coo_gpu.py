"""COO (the reference's COOMatrix, src/formats/sparse_formats.h:113-162,
declared there without a kernel): the device conversion to CSR is bit-exact
against a numpy stable (row, column) ordering, and SpMV on COO matches the
FP64 oracle on that CSR (bound 1e-5 FP32 / 1e-13 FP64 times sum |a x|)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import tol_for

pytestmark = pytest.mark.gpu


def np_coo_to_csr(ri, ci, v, R):
    order = np.lexsort((ci, ri))  # by row, then column; stable for equal pairs
    rp = np.zeros(R + 1, np.int64)
    np.add.at(rp, ri.astype(np.int64) + 1, 1)
    return np.cumsum(rp).astype(np.int32), ci[order], v[order]


def cases():
    rng = np.random.default_rng(12)
    out = {}
    R, C, n = 7000, 5000, 60000
    out["shuffled"] = (rng.integers(0, R, n).astype(np.int32), rng.integers(0, C, n).astype(np.int32),
                       rng.standard_normal(n), R, C)
    ri = np.repeat(np.arange(50, dtype=np.int32), 3)
    ci = np.tile(np.array([4, 4, 1], np.int32), 50)  # duplicate (row, col) pairs
    out["duplicates"] = (ri[::-1].copy(), ci[::-1].copy(), rng.standard_normal(150), 60, 10)
    out["one_long_row"] = (np.full(40000, 3, np.int32), rng.integers(0, 90000, 40000).astype(np.int32),
                           rng.standard_normal(40000), 9, 90000)
    out["empty"] = (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0), 5, 5)
    return out


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_coo_to_csr_bit_exact(mx, cuda, dtype):
    for name, (ri, ci, v, R, C) in cases().items():
        A = mx.COOMatrix(ri, ci, v.astype(dtype), R, C).copyToDevice()
        B = mx.coo_to_csr(A)
        cuda.cuda.synchronize()
        rp, cs, vs = np_coo_to_csr(ri, ci, v.astype(dtype), R)
        assert np.array_equal(B.d_rowPtr.cpu().numpy(), rp), name
        assert np.array_equal(B.d_colIdx.cpu().numpy()[:len(cs)], cs), name
        assert np.array_equal(B.d_values.cpu().numpy()[:len(vs)], vs), name


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_coo_spmv_matches_oracle(mx, cuda, dtype):
    for name, (ri, ci, v, R, C) in cases().items():
        v = v.astype(dtype)
        A = mx.COOMatrix(ri, ci, v, R, C).copyToDevice()
        rp, cs, vs = np_coo_to_csr(ri, ci, v, R)
        xh = mx.gen_vector(C, 5, dtype=dtype)
        y_ref, absum = oracle.spmv_ref(rp, cs, vs, xh)
        for alpha, beta in ((1.0, 0.0), (0.5, -2.0)):
            y0 = mx.gen_vector(R, 6, dtype=dtype)
            y = cuda.from_numpy(y0.copy()).cuda()
            mx.spmv_coo(A, cuda.from_numpy(xh).cuda(), y, alpha, beta)
            cuda.cuda.synchronize()
            want = alpha * y_ref + beta * y0.astype(np.float64)
            bound = tol_for(dtype) * (abs(alpha) * absum + abs(beta * y0.astype(np.float64)))
            got = y.cpu().numpy().astype(np.float64)
            assert (np.abs(got - want) <= bound + (0 if dtype == np.float64 else 1e-30)).all(), (name, alpha)


def test_coo_out_of_range_refused(mx, cuda):
    ri = np.array([0, 1, 5], np.int32)  # row 5 of a 5-row matrix
    ci = np.array([0, 1, 2], np.int32)
    A = mx.COOMatrix(ri, ci, np.ones(3, np.float32), 5, 5).copyToDevice()
    with pytest.raises(mx.SpmvError) as e:
        mx.coo_to_csr(A)
    assert e.value.status == -2
    ci2 = np.array([0, -1, 2], np.int32)
    B = mx.COOMatrix(np.zeros(3, np.int32), ci2, np.ones(3, np.float32), 5, 5).copyToDevice()
    with pytest.raises(mx.SpmvError):
        mx.spmv_coo(B, cuda.ones(5, device="cuda"), cuda.zeros(5, device="cuda"))
