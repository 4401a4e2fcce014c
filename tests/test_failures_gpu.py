"""Out-of-memory paths, by injection on the host (spmv_debug_fail_allocation):
for each call that allocates device memory -- plans of every kind, the
transposed plan built on first use, plans that copy the matrix, pipelines,
batches, selector models and the stateless call's scratch -- the n-th
allocation is made to fail for n = 1, 2, ... until the call succeeds.  Every
failing attempt must return SPMV_ERROR_MEMORY_ALLOC (the reference's status
value, src/utils/common.h:31-43) and leave the library's live device memory
exactly where it was; the attempt that succeeds must give the oracle's
result.  No GPU fault is involved: the CUDA driver is never asked for the failing
allocation."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import device_csr

pytestmark = pytest.mark.gpu
MEMORY_ALLOC = -4


@pytest.fixture(scope="module")
def mat(mx):
    from muxi_spmv_gb300 import workloads as W
    s = W.scaled("powerlaw8m", 30000, seed=11)
    rp, ci, v = mx.generate(s)
    return rp, ci, v, s.numCols


def _each_failure(mx, torch, make, use=None, max_tries=40):
    """Runs make() with the n-th allocation failing, n = 1.. until it
    succeeds; returns (failures seen, the successful result)."""
    base = mx.debug_device_memory()
    for n in range(1, max_tries + 1):
        mx.debug_fail_allocation(n)
        try:
            obj = make()
        except mx.SpmvError as e:
            mx.debug_fail_allocation(0)
            torch.cuda.synchronize()
            assert e.status == MEMORY_ALLOC, f"allocation {n}: {e}"
            assert mx.debug_device_memory() == base, f"allocation {n} failed but device memory leaked"
            continue
        mx.debug_fail_allocation(0)
        return n - 1, obj, base
    mx.debug_fail_allocation(0)
    raise AssertionError("the call still failed after injecting into every allocation tried")


def _check(mx, y, rp, ci, v, xh):
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    r = oracle.row_errors(y.cpu().numpy(), y_ref, absum, 1e-5)
    assert np.all(r <= 1.0)


@pytest.mark.parametrize("kind", ["auto", "merge", "ell", "band", "copy", "rows"])
def test_plan_creation_out_of_memory(mx, cuda, handle, mat, kind):
    torch = cuda
    rp, ci, v, cols = mat
    A = device_csr(mx, rp, ci, v, cols)
    variant = {"auto": None, "merge": mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4),
               "ell": mx.make_variant(mx.KERNEL_ELL), "band": mx.make_variant(mx.KERNEL_BAND, 512, 0, 16, 0),
               "copy": None, "rows": mx.make_variant(mx.KERNEL_VECTOR, 256, 8, 0, 4)}[kind]
    if kind == "ell":  # a stencil: ELL refuses the power-law matrix's padding
        from muxi_spmv_gb300 import workloads as W
        s = W.scaled("stencil2d_4096", 10000, 3)
        rp, ci, v = mx.generate(s)
        cols = s.numCols
        A = device_csr(mx, rp, ci, v, cols)
    fails, p, base = _each_failure(mx, torch, lambda: mx.Plan(handle, A, variant, copy=(kind == "copy")))
    if kind != "rows":  # row kernels keep no device state
        assert fails >= 1
    xh = mx.gen_vector(cols, 3)
    x = torch.from_numpy(xh).cuda()
    y = torch.empty(A.numRows, device="cuda")
    p.exec(x, y)
    torch.cuda.synchronize()
    _check(mx, y, rp, ci, v, xh)
    p.destroy()
    assert mx.debug_device_memory() == base


def test_transposed_plan_out_of_memory(mx, cuda, handle, mat):
    """The first transposed execution builds A^T and its plan: an allocation
    failing there fails that execution only, and the next one succeeds."""
    torch = cuda
    rp, ci, v, cols = mat
    A = device_csr(mx, rp, ci, v, cols)
    p = mx.Plan(handle, A)
    yh = mx.gen_vector(A.numRows, 4)
    yt = torch.from_numpy(yh).cuda()
    out = torch.empty(cols, device="cuda")
    fails, _, _ = _each_failure(mx, torch, lambda: p.exec(yt, out, transpose=True))
    assert fails >= 1
    torch.cuda.synchronize()
    # A^T y against the oracle on the transposed CSR
    import scipy.sparse as sp
    At = sp.csr_matrix((v, ci, rp), shape=(A.numRows, cols)).T.tocsr()
    At.sort_indices()
    ref, absum = oracle.spmv_ref(At.indptr.astype(np.int32), At.indices.astype(np.int32),
                                 At.data.astype(np.float32), yh)
    assert np.all(oracle.row_errors(out.cpu().numpy(), ref, absum, 1e-5) <= 1.0)
    p.destroy()


def test_pipeline_out_of_memory(mx, cuda, handle, mat):
    torch = cuda
    rp, ci, v, cols = mat
    A = device_csr(mx, rp, ci, v, cols)
    fails, pipe, base = _each_failure(mx, torch, lambda: mx.Pipeline(handle, A, slices=4, depth=2))
    assert fails >= 3
    xh = mx.gen_vector(cols, 5)
    y = torch.empty(A.numRows).pin_memory()
    pipe.submit(torch.from_numpy(xh).pin_memory(), y)
    pipe.wait()
    _check(mx, y, rp, ci, v, xh)
    pipe.destroy()
    assert mx.debug_device_memory() == base


def test_batch_out_of_memory(mx, cuda, handle):
    torch = cuda
    from muxi_spmv_gb300 import batch as B
    from muxi_spmv_gb300 import selector as S
    mats = [S.gen_device(mx.GenSpec(mx.GEN_POISSON_UNIFORM, r, r, 9.0, 40.0, 0.0, 0.0, 40 + i))
            for i, r in enumerate((3000, 17000, 1200))]
    torch.cuda.synchronize()
    fails, plan, base = _each_failure(mx, torch, lambda: B.BatchPlan(handle, mats, 2))
    assert fails >= 1
    xs = [torch.rand(A.numCols * 2, device="cuda") for A in mats]
    ys = [torch.empty(A.numRows * 2, device="cuda") for A in mats]
    plan.set_vectors(xs, ys)
    plan.exec(1.0, 0.0, B.BATCH_PERSISTENT)
    torch.cuda.synchronize()
    for A, X, Y in zip(mats, xs, ys):
        rp, ci = A.d_rowPtr.cpu().numpy(), A.d_colIdx[:A.nnz].cpu().numpy()
        vv = A.d_values[:A.nnz].cpu().numpy()
        Xh, Yh = X.cpu().numpy().reshape(A.numCols, 2), Y.cpu().numpy().reshape(A.numRows, 2)
        for j in range(2):
            ref, absum = oracle.spmv_ref(rp, ci, vv, np.ascontiguousarray(Xh[:, j]))
            assert np.all(oracle.row_errors(Yh[:, j], ref, absum, 1e-5) <= 1.0)
    plan.destroy()
    assert mx.debug_device_memory() == base


def test_stateless_scratch_and_model_out_of_memory(mx, cuda, mat):
    torch = cuda
    rp, ci, v, cols = mat
    A = device_csr(mx, rp, ci, v, cols)
    xh = mx.gen_vector(cols, 6)
    x = torch.from_numpy(xh).cuda()
    y = torch.empty(A.numRows, device="cuda")
    fails, _, base = _each_failure(mx, torch, lambda: mx.spmv_csr(A, x, y))
    assert fails >= 1
    torch.cuda.synchronize()
    _check(mx, y, rp, ci, v, xh)
    from muxi_spmv_gb300 import selector as S
    fails, model, base = _each_failure(mx, torch, lambda: S.MLP.load(S.DEFAULT_MODEL))
    assert fails >= 1
    model.destroy()
    assert mx.debug_device_memory() == base
