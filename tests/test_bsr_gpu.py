"""BSR (the reference's BSRMatrix, src/formats/sparse_formats.h:207-269,
declared there without a conversion or kernel): the device CSR->BSR
conversion equals a numpy construction of the same blocks bit for bit, and
the BSR SpMV matches the FP64 oracle on the CSR (bound 1e-5 FP32 / 1e-13 FP64
times sum |a x|, plus |beta*y0|)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu


def np_bsr(rp, ci, v, R, C, B):
    nbr = (R + B - 1) // B
    rows = np.repeat(np.arange(R), np.diff(rp))
    keys = sorted({(r // B, c // B) for r, c in zip(rows.tolist(), ci.tolist())})
    brp = np.zeros(nbr + 1, np.int64)
    for br, _ in keys:
        brp[br + 1] += 1
    brp = np.cumsum(brp).astype(np.int32)
    bci = np.array([bc for _, bc in keys], np.int32)
    index = {k: i for i, k in enumerate(keys)}
    vals = np.zeros((len(keys), B, B), v.dtype)
    for r, c, a in zip(rows.tolist(), ci.tolist(), v.tolist()):
        vals[index[(r // B, c // B)], r % B, c % B] += a
    return brp, bci, vals.reshape(-1)


def cases():
    rng = np.random.default_rng(9)
    out = {}
    # block-structured (FEM-like): dense B x B blocks on a banded block pattern, R and C not multiples of B
    R, C = 1003, 997
    lens = rng.integers(0, 12, R)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    ci = np.concatenate([np.sort(rng.choice(C, l, replace=False)) for l in lens]).astype(np.int32)
    out["random"] = (rp, ci, rng.standard_normal(rp[-1]), R, C)
    # near-diagonal rows with a long one and empty block rows
    lens = np.r_[rng.integers(1, 6, 500), 0, 0, 0, 0, 0, 0, 0, 0, 3000, rng.integers(0, 4, 300)].astype(np.int32)
    R = len(lens)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    C = 4000
    ci = np.concatenate([np.sort(rng.choice(C, l, replace=False)) for l in lens]).astype(np.int32)
    out["longrow_empty"] = (rp, ci, rng.standard_normal(rp[-1]), R, C)
    out["no_nnz"] = (np.zeros(10, np.int32), np.zeros(0, np.int32), np.zeros(0), 9, 7)
    return out


@pytest.mark.parametrize("B", [2, 4, 8])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_bsr_conversion_and_spmv(mx, cuda, B, dtype):
    for name, (rp, ci, v, R, C) in cases().items():
        v = v.astype(dtype)
        A = device_csr(mx, rp, ci, v, C)
        M = mx.csr_to_bsr(A, B)
        cuda.cuda.synchronize()
        brp, bci, bv = np_bsr(rp, ci, v, R, C, B)
        assert M.numBlocks == len(bci), name
        assert np.array_equal(M.d_rowPtr.cpu().numpy(), brp), name
        assert np.array_equal(M.d_colIdx.cpu().numpy()[:len(bci)], bci), name
        assert np.array_equal(M.d_values.cpu().numpy()[:len(bv)], bv), name
        xh = mx.gen_vector(C, 4, dtype=dtype)
        y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
        for alpha, beta in ((1.0, 0.0), (-0.75, 1.5)):
            y0 = mx.gen_vector(R, 5, dtype=dtype)
            y = cuda.from_numpy(y0.copy()).cuda()
            mx.spmv_bsr(M, cuda.from_numpy(xh).cuda(), y, alpha, beta)
            cuda.cuda.synchronize()
            want = alpha * y_ref + beta * y0.astype(np.float64)
            bound = tol_for(dtype) * (abs(alpha) * absum + abs(beta * y0.astype(np.float64)))
            got = y.cpu().numpy().astype(np.float64)
            assert (np.abs(got - want) <= bound + (0 if dtype == np.float64 else 1e-30)).all(), (name, B, alpha)


def test_bsr_refuses_unsorted_rows_and_bad_block_size(mx, cuda):
    rp = np.array([0, 3], np.int32)
    ci = np.array([5, 1, 2], np.int32)  # unsorted
    A = device_csr(mx, rp, ci, np.ones(3, np.float32), 8)
    with pytest.raises(mx.SpmvError) as e:
        mx.csr_to_bsr(A, 4)
    assert e.value.status == -2
    A2 = device_csr(mx, rp, np.sort(ci), np.ones(3, np.float32), 8)
    with pytest.raises(mx.SpmvError):
        mx.csr_to_bsr(A2, 3)
