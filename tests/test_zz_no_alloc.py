"""spmv_csr_noalloc_f32, the entry point for callers that cannot allocate
device memory (graph recording, externally owned memory budgets, real-time
loops).  Called through the C ABI twice in a row, on different matrices, its
output must match spmv_csr_f32's within the FP32 row bound; a matrix too large
for its fixed scratch array is rejected.  This file is collected last so a
failing run that stops at the first failure has already run everything else."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _call(mx, A, x, y, alpha, beta, stream):
    return mx.lib().spmv_csr_noalloc_f32(A.numRows, A.numCols, A.nnz, A.d_rowPtr.data_ptr(), A.d_colIdx.data_ptr(),
                                         A.d_values.data_ptr(), x.data_ptr(), y.data_ptr(), alpha, beta, stream)


def test_noalloc_matches_spmv_csr_two_calls(mx, cuda):
    torch = cuda
    from muxi_spmv_gb300 import workloads as W
    stream = torch.cuda.current_stream().cuda_stream or None
    mats = []
    for name, rows, seed in (("powerlaw8m", 150000, 31), ("poisson16k", 16384, 32)):
        s = W.scaled(name, rows, seed) if name != "poisson16k" else W.spec(name, seed)
        rp, ci, v = mx.generate(s)
        A = mx.CSRMatrix(rp, ci, v, s.numCols).copyToDevice()
        mats.append(A)
    for A, (alpha, beta) in zip(mats, ((1.0, 0.0), (0.75, -1.25))):
        xh = mx.gen_vector(A.numCols, 5)
        x = torch.from_numpy(xh).cuda()
        y0 = mx.gen_vector(A.numRows, 6)
        y_ref_dev = torch.from_numpy(y0.copy()).cuda()
        mx.spmv_csr(A, x, y_ref_dev, alpha, beta)
        y = torch.from_numpy(y0.copy()).cuda()
        st = _call(mx, A, x, y, alpha, beta, stream)
        assert st == 0, mx.last_error()
        torch.cuda.synchronize()
        got, want = y.cpu().numpy().astype(np.float64), y_ref_dev.cpu().numpy().astype(np.float64)
        _, absum = oracle.spmv_ref(A.rowPtr, A.colIdx, A.values, xh)
        scale = abs(alpha) * absum + abs(beta) * np.abs(y0.astype(np.float64))
        bound = 1e-5 * scale + 2 * np.finfo(np.float32).eps * np.abs(want)
        assert np.all(np.abs(got - want) <= bound)


def test_noalloc_rejects_oversize(mx, cuda):
    # Sizes beyond the fixed scratch are refused before any device access.
    L = mx.lib()
    bogus = C.c_void_p(16)
    st = L.spmv_csr_noalloc_f32(2_000_000_000, 10, 2_000_000_000, bogus, bogus, bogus, bogus, bogus, 1.0, 0.0, None)
    assert st == -4
    assert "no-allocation" in mx.last_error()
