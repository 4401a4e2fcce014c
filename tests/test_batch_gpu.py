"""GPU parity of the batched SpMV / SpMM (spmv_batch_*) against the FP64
oracle, column by column: |Y - (alpha*A*X + beta*Y0)| <= 1e-5 * (|alpha|
sum_j |a_ij x_j| + |beta*Y0|) per row and column, for every execution mode,
k in {1, 2, 4, 8, 16}, and batches with empty matrices, matrices without
rows, and rows spanning many tiles and many warps' tile ranges."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _host_batch(mx):
    from muxi_spmv_gb300 import workloads as W
    rng = np.random.default_rng(21)
    mats = []
    # regular and power-law matrices of uneven sizes
    for i in range(24):
        R = int(np.exp(rng.uniform(np.log(300), np.log(120000))))
        if i % 3 == 0:
            s = W.scaled("powerlaw8m", R, seed=100 + i)
        else:
            s = mx.GenSpec(mx.GEN_POISSON_UNIFORM, R, R, float(rng.uniform(2, 40)), 0.0, 200.0, 0.0, 200 + i)
        rp, ci, v = mx.generate(s)
        mats.append((rp, ci, v, s.numCols))
    # one row of 2,000,000 nonzeros among short rows (spans thousands of tiles)
    lens = np.r_[rng.integers(0, 5, 200), 2_000_000, rng.integers(0, 5, 300)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    cols = 90000
    ci = rng.integers(0, cols, rp[-1]).astype(np.int32)
    ci = np.concatenate([np.sort(ci[rp[r]:rp[r + 1]]) for r in range(len(lens))])
    mats.insert(5, (rp, ci, rng.standard_normal(rp[-1]).astype(np.float32), cols))
    # a 65,536-nonzero row
    lens = np.r_[rng.integers(0, 3, 100), 65536, rng.integers(0, 3, 100)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    mats.insert(9, (rp, np.sort(rng.integers(0, 70000, rp[-1])).astype(np.int32),
                    rng.standard_normal(rp[-1]).astype(np.float32), 70000))
    # no nonzeros; no rows; one row; empty rows at both ends
    mats.insert(0, (np.zeros(51, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 40))
    mats.insert(12, (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 10))
    mats.append((np.array([0, 3], np.int32), np.array([0, 4, 4], np.int32), np.array([1, 2, 3], np.float32), 6))
    lens = np.r_[np.zeros(30), rng.integers(0, 3, 500), np.zeros(40)].astype(np.int32)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    mats.append((rp, rng.integers(0, 77, rp[-1]).astype(np.int32), rng.standard_normal(rp[-1]).astype(np.float32),
                 77))
    return mats


@pytest.fixture(scope="module")
def hbatch(mx, cuda):
    return _host_batch(mx)


@pytest.fixture(scope="module")
def dmats(mx, cuda, hbatch):
    return [mx.CSRMatrix(rp, ci, v, c).copyToDevice() for rp, ci, v, c in hbatch]


def _check(hbatch, X, Y0, Y, k, alpha, beta):
    worst = 0.0
    for (rp, ci, v, c), x, y0, y in zip(hbatch, X, Y0, Y):
        R = len(rp) - 1
        if R == 0:
            continue
        y = y.reshape(R, k)
        y0 = y0.reshape(R, k)
        for j in range(k):
            yr, absum = oracle.spmv_ref(rp, ci, v, np.ascontiguousarray(x.reshape(c, k)[:, j]))
            want = alpha * yr + beta * y0[:, j].astype(np.float64)
            bound = 1e-5 * (abs(alpha) * absum + abs(beta * y0[:, j].astype(np.float64)))
            err = np.abs(y[:, j].astype(np.float64) - want)
            ok = err <= bound
            assert ok.all(), f"k={k} col {j}: {int((~ok).sum())} rows off, worst {err[~ok].max()}"
            worst = max(worst, float((err / np.where(bound > 0, bound, 1)).max()))
    return worst


@pytest.mark.parametrize("k", [1, 2, 4, 8, 16])
def test_batch_matches_oracle_all_modes(mx, cuda, handle, hbatch, dmats, k):
    from muxi_spmv_gb300 import batch as B
    rng = np.random.default_rng(k)
    X = [rng.uniform(-1, 1, c * k).astype(np.float32) for (_, _, _, c) in hbatch]
    Y0 = [rng.uniform(-1, 1, (len(rp) - 1) * k).astype(np.float32) for (rp, _, _, _) in hbatch]
    dX = [cuda.from_numpy(x).cuda() if x.size else cuda.zeros(4, device="cuda") for x in X]
    plan = B.BatchPlan(handle, dmats, k)
    info = plan.info()
    assert info["nnz"] == sum(int(rp[-1]) for rp, *_ in hbatch)
    assert info["tiles"] > 4 * info["warps"]  # warps chain several tiles each
    outs = {}
    for mode in (B.BATCH_PERSISTENT, B.BATCH_PERSISTENT_GRAPH, B.BATCH_LOOP, B.BATCH_LOOP_GRAPH):
        for alpha, beta in ((1.0, 0.0), (1.5, -0.5)):
            dY = [cuda.from_numpy(y0.copy()).cuda() if y0.size else cuda.zeros(4, device="cuda") for y0 in Y0]
            plan.set_vectors(dX, dY)
            plan.exec(alpha, beta, mode)
            cuda.cuda.synchronize()
            Y = [y.cpu().numpy()[:y0.size] for y, y0 in zip(dY, Y0)]
            _check(hbatch, X, Y0, Y, k, alpha, beta)
            outs[(mode, alpha)] = Y
    # replaying the same mode gives bit-identical results (no atomics)
    dY = [cuda.from_numpy(y0.copy()).cuda() if y0.size else cuda.zeros(4, device="cuda") for y0 in Y0]
    plan.set_vectors(dX, dY)
    for _ in range(3):
        plan.exec(1.0, 0.0, B.BATCH_PERSISTENT_GRAPH)
    cuda.cuda.synchronize()
    for a, b in zip(outs[(B.BATCH_PERSISTENT_GRAPH, 1.0)], [y.cpu().numpy() for y in dY]):
        assert np.array_equal(a, b[:a.size])
    plan.destroy()


def test_batch_group_mixed_k_matches_oracle(mx, cuda, handle, hbatch, dmats):
    """A group whose matrices carry their own k (all five values mixed), in
    every mode, against the oracle column by column; the same matrices as
    single-k batches give the same bits."""
    from muxi_spmv_gb300 import batch as B
    rng = np.random.default_rng(77)
    ks = [int(k) for k in rng.choice([1, 2, 4, 8, 16], len(hbatch))]
    X = [rng.uniform(-1, 1, c * k).astype(np.float32) for (_, _, _, c), k in zip(hbatch, ks)]
    Y0 = [rng.uniform(-1, 1, (len(rp) - 1) * k).astype(np.float32) for (rp, *_), k in zip(hbatch, ks)]
    dX = [cuda.from_numpy(x).cuda() if x.size else cuda.zeros(4, device="cuda") for x in X]
    g = B.BatchGroupPlan(handle, dmats, ks)
    assert g.info()["batches"] == len(set(ks))
    for mode in (B.BATCH_PERSISTENT, B.BATCH_PERSISTENT_GRAPH, B.BATCH_LOOP, B.BATCH_LOOP_GRAPH):
        dY = [cuda.from_numpy(y0.copy()).cuda() if y0.size else cuda.zeros(4, device="cuda") for y0 in Y0]
        g.set_vectors(dX, dY)
        g.exec(1.5, -0.5, mode)
        cuda.cuda.synchronize()
        Y = [y.cpu().numpy()[:y0.size] for y, y0 in zip(dY, Y0)]
        for i, k in enumerate(ks):
            _check([hbatch[i]], [X[i]], [Y0[i]], [Y[i]], k, 1.5, -0.5)
    # one single-k batch of the k = 4 members reproduces their bits
    dY = [cuda.from_numpy(y0.copy()).cuda() if y0.size else cuda.zeros(4, device="cuda") for y0 in Y0]
    g.set_vectors(dX, dY)
    g.exec(1.5, -0.5, B.BATCH_PERSISTENT_GRAPH)
    cuda.cuda.synchronize()
    Y = [y.cpu().numpy()[:y0.size] for y, y0 in zip(dY, Y0)]
    idx = [i for i, k in enumerate(ks) if k == 4]
    if idx:
        p = B.BatchPlan(handle, [dmats[i] for i in idx], 4)
        dY2 = [cuda.from_numpy(Y0[i].copy()).cuda() if Y0[i].size else cuda.zeros(4, device="cuda") for i in idx]
        p.set_vectors([dX[i] for i in idx], dY2)
        p.exec(1.5, -0.5, B.BATCH_PERSISTENT_GRAPH)
        cuda.cuda.synchronize()
        for i, y2 in zip(idx, dY2):
            assert np.array_equal(Y[i], y2.cpu().numpy()[:Y0[i].size])
        p.destroy()
    with pytest.raises(mx.SpmvError):
        B.BatchGroupPlan(handle, dmats[:2], [1, 3])
    g.destroy()


def test_batch_rejects_bad_input(mx, cuda, handle, dmats):
    from muxi_spmv_gb300 import batch as B
    with pytest.raises(mx.SpmvError):
        B.BatchPlan(handle, dmats[:3], 3)  # k not in {1,2,4,8,16}
    plan = B.BatchPlan(handle, dmats[:3], 4)
    with pytest.raises(mx.SpmvError):
        plan.exec()  # vectors not bound
    xs = [cuda.zeros(A.numCols * 4 + 1, device="cuda")[1:] for A in dmats[:3]]  # misaligned
    ys = [cuda.zeros(max(A.numRows * 4, 1), device="cuda") for A in dmats[:3]]
    with pytest.raises(mx.SpmvError, match="aligned"):
        plan.set_vectors(xs, ys)
    plan.destroy()


def test_uneven_batch_small_sample(mx, cuda, handle):
    """The uneven-batch workload's generator at reduced size: structure and
    a persistent-vs-oracle check on two sampled matrices."""
    from muxi_spmv_gb300 import batch as B
    mats, xs, ys, specs = B.build_uneven_batch(count=24, k=4, seed=3, rmax=20000)
    for A, s in zip(mats, specs):
        assert A.numRows == s.spec.numRows and mx.validate_csr(A) == 0
        mean = A.nnz / A.numRows
        if s.law == "poisson":
            assert abs(mean - s.mean_target) < 0.2 * s.mean_target + 1
    plan = B.BatchPlan(handle, mats, 4)
    plan.set_vectors(xs, ys)
    plan.exec(1.0, 0.0, B.BATCH_PERSISTENT_GRAPH)
    cuda.cuda.synchronize()
    for i in (0, 17):
        A = mats[i]
        rp, ci, v = (t.cpu().numpy() for t in (A.d_rowPtr, A.d_colIdx, A.d_values))
        ci, v = ci[:A.nnz], v[:A.nnz]
        X = xs[i].cpu().numpy().reshape(A.numCols, 4)
        Y = ys[i].cpu().numpy()[:A.numRows * 4].reshape(A.numRows, 4)
        for j in range(4):
            yr, absum = oracle.spmv_ref(rp, ci, v, np.ascontiguousarray(X[:, j]))
            assert (np.abs(Y[:, j] - yr) <= 1e-5 * absum).all()


@pytest.mark.parametrize("k,variant", [(1, {"nnzPerSlot": 4, "blocksPerSM": 3, "chunkNnz": 1024}),
                                       (2, {"nnzPerSlot": 4, "blocksPerSM": 2, "chunkNnz": 4096}),
                                       (1, {"nnzPerSlot": 8, "blocksPerSM": 2, "chunkNnz": 256}),
                                       (16, {"nnzPerSlot": 4, "blocksPerSM": 3, "chunkNnz": 32}),
                                       (1, {"nnzPerSlot": 16, "blocksPerSM": 10, "ordered": 1}),
                                       (1, {"nnzPerSlot": 8, "blocksPerSM": 12, "ordered": 1})])
def test_batch_variants_match_oracle(mx, cuda, handle, hbatch, dmats, k, variant):
    """Every launch shape, including the ordered k = 1 tiles (one warp per
    CSR5 tile, per-tile carries joined across tiles of one matrix only), on
    the batch with empty matrices, a matrix without rows and rows over
    thousands of tiles; alpha/beta and the plain y = A x epilogue."""
    from muxi_spmv_gb300 import batch as B
    rng = np.random.default_rng(100 + k)
    X = [rng.uniform(-1, 1, c * k).astype(np.float32) for (_, _, _, c) in hbatch]
    Y0 = [rng.uniform(-1, 1, (len(rp) - 1) * k).astype(np.float32) for (rp, _, _, _) in hbatch]
    dX = [cuda.from_numpy(x).cuda() for x in X]
    plan = B.BatchPlan(handle, dmats, k, variant)
    want = {"chunkNnz": 0, "ordered": 0, **variant}
    if want["ordered"]:
        want["chunkNnz"] = 32 * want["nnzPerSlot"]  # one tile per warp
    assert plan.variant == want
    for mode in (B.BATCH_PERSISTENT_GRAPH, B.BATCH_LOOP):
        for alpha, beta in ((0.75, 0.25), (1.0, 0.0)):
            dY = [cuda.from_numpy(y0.copy()).cuda() if y0.size else cuda.zeros(4, device="cuda") for y0 in Y0]
            plan.set_vectors(dX, dY)
            plan.exec(alpha, beta, mode)
            cuda.cuda.synchronize()
            _check(hbatch, X, Y0, [y.cpu().numpy()[:y0.size] for y, y0 in zip(dY, Y0)], k, alpha, beta)
    plan.destroy()
    with pytest.raises(mx.SpmvError):
        B.BatchPlan(handle, dmats, 2, {"ordered": 1})  # ordered tiles serve k = 1 only
    with pytest.raises(mx.SpmvError):
        B.BatchPlan(handle, dmats, 4, {"nnzPerSlot": 8, "blocksPerSM": 3})  # not built
    with pytest.raises(mx.SpmvError):
        B.BatchPlan(handle, dmats, 1, {"chunkNnz": 300})  # not a multiple of the tile
