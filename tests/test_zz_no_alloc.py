"""spmv_csr_noalloc_f32, the entry point for callers that cannot allocate
device memory (a memory budget owned by another allocator, a real-time loop
that must not pay for an allocation).  Called through the C ABI twice in a
row, on different matrices, its output must match spmv_csr_f32's (the
existing entry point) and the FP64 oracle within the FP32 row bound, also
when colIdx / values are not 16-byte aligned; a matrix too large for its fixed
scratch array is rejected with a message that states the limit.  This file
is collected last so a failing run that stops at the first failure has
already run everything else."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _call(mx, A, x, y, alpha, beta, stream, ci=None, v=None):
    ci = A.d_colIdx if ci is None else ci
    v = A.d_values if v is None else v
    return mx.lib().spmv_csr_noalloc_f32(A.numRows, A.numCols, A.nnz, A.d_rowPtr.data_ptr(), ci.data_ptr(),
                                         v.data_ptr(), x.data_ptr(), y.data_ptr(), alpha, beta, stream)


def _bound(absum, y0, want, alpha, beta):
    """|y - y_ref| <= 1e-5 * sum|a x| for y = A x; with alpha != 1 or beta != 0
    the scaled terms and one FP32 rounding of the epilogue are added."""
    if alpha == 1.0 and beta == 0.0:
        return 1e-5 * absum
    scale = abs(alpha) * absum + abs(beta) * np.abs(y0.astype(np.float64))
    return 1e-5 * scale + 2 * np.finfo(np.float32).eps * np.abs(want)


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
        y_dev = torch.from_numpy(y0.copy()).cuda()
        mx.spmv_csr(A, x, y_dev, alpha, beta)  # the existing entry point
        y = torch.from_numpy(y0.copy()).cuda()
        st = _call(mx, A, x, y, alpha, beta, stream)
        assert st == 0, mx.last_error()
        torch.cuda.synchronize()
        got, existing = y.cpu().numpy().astype(np.float64), y_dev.cpu().numpy().astype(np.float64)
        y_ref, absum = oracle.spmv_ref(A.rowPtr, A.colIdx, A.values, xh)
        want = alpha * y_ref + beta * y0.astype(np.float64)
        bound = _bound(absum, y0, want, alpha, beta)
        assert np.all(np.abs(got - want) <= bound), "no-allocation call against the FP64 oracle"
        assert np.all(np.abs(got - existing) <= 2 * bound), "no-allocation call against spmv_csr_f32"


def test_noalloc_unaligned_arrays(mx, cuda):
    """colIdx and values one element past a 16-byte boundary: the per-item
    merge tiles run instead of the 16-byte loads."""
    torch = cuda
    from muxi_spmv_gb300 import workloads as W
    s = W.scaled("powerlaw8m", 40000, 33)
    rp, ci, v = mx.generate(s)
    A = mx.CSRMatrix(rp, ci, v, s.numCols).copyToDevice()
    ci_buf = torch.zeros(A.nnz + 4, dtype=torch.int32, device="cuda")
    v_buf = torch.zeros(A.nnz + 4, dtype=torch.float32, device="cuda")
    ci_u, v_u = ci_buf[1:A.nnz + 1], v_buf[1:A.nnz + 1]
    ci_u.copy_(A.d_colIdx[:A.nnz])
    v_u.copy_(A.d_values[:A.nnz])
    assert ci_u.data_ptr() % 16 != 0 and v_u.data_ptr() % 16 != 0
    xh = mx.gen_vector(A.numCols, 7)
    x = torch.from_numpy(xh).cuda()
    y = torch.empty(A.numRows, device="cuda")
    st = _call(mx, A, x, y, 1.0, 0.0, torch.cuda.current_stream().cuda_stream or None, ci_u, v_u)
    assert st == 0, mx.last_error()
    torch.cuda.synchronize()
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    assert np.all(np.abs(y.cpu().numpy().astype(np.float64) - y_ref) <= 1e-5 * absum)


def test_noalloc_rejects_oversize(mx, cuda):
    # Sizes beyond the fixed scratch are refused before any device access.
    L = mx.lib()
    bogus = C.c_void_p(16)
    st = L.spmv_csr_noalloc_f32(2_000_000_000, 10, 2_000_000_000, bogus, bogus, bogus, bogus, bogus, 1.0, 0.0, None)
    assert st == -4
    msg = mx.last_error()
    assert "no-allocation" in msg and "up to 1071" in msg  # 16-byte-aligned arrays: about 1.07e9
