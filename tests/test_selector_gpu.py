"""GPU checks of the learned-selector stack through the C ABI: the device
generators, the feature kernel (against a numpy restatement), the MLP's CUDA
forward / gradients / Adam (against the FP64 numpy restatement in
mlp_ref.py), the model file, the autotuner, spmv_select and AUTO plans with
a registered model (parity against the FP64 oracle)."""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import pytest

import mlp_ref
import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sel(mx, cuda):
    from muxi_spmv_gb300 import selector
    return selector


def host(t):
    return t.cpu().numpy()


# ---------------------------------------------------------------------------
# device generators
# ---------------------------------------------------------------------------
def _gen(mx, sel, kind, R, p0, p1=0.0, p2=0.0, seed=7, C=None):
    spec = mx.GenSpec(kind, R, C or R, p0, p1, p2, 0.0, seed)
    return spec, sel.gen_device(spec)


@pytest.mark.parametrize("law", ["poisson", "zipf", "banded", "blockdiag"])
def test_device_generator_laws(mx, sel, cuda, law):
    R = 30000
    if law == "poisson":
        spec, A = _gen(mx, sel, mx.GEN_POISSON_UNIFORM, R, 12.0, 0.0, 64.0)
    elif law == "zipf":
        spec, A = _gen(mx, sel, mx.GEN_ZIPF_UNIFORM, R, 1.8, 4096.0)
    elif law == "banded":
        spec, A = _gen(mx, sel, mx.GEN_BANDED, R, 20.0, 65.0)
    else:
        spec, A = _gen(mx, sel, mx.GEN_BLOCKDIAG, R, 16.0, 30.0)
    cuda.cuda.synchronize()
    assert mx.validate_csr(A) == 0
    rp, ci = host(A.d_rowPtr), host(A.d_colIdx)[:A.nnz]
    assert rp[0] == 0 and rp[-1] == A.nnz
    lens = np.diff(rp)
    rows = np.repeat(np.arange(R), lens)
    # sorted within each row (repeats allowed)
    d = np.diff(ci.astype(np.int64))
    same_row = rows[1:] == rows[:-1]
    assert (d[same_row] >= 0).all()
    if law == "poisson":
        assert abs(lens.mean() - 12.0) < 0.3 and lens.max() <= 64
    if law == "zipf":
        assert lens.min() >= 1 and lens.max() <= 4096
    if law == "banded":
        w = 65
        lo = np.clip(rows - w // 2, 0, R - w)
        assert (ci >= lo).all() and (ci < lo + w).all()
        assert lens.min() >= 1 and lens.max() <= w
    if law == "blockdiag":
        b = rows.astype(np.int64) * 16 // R
        assert (ci >= b * R // 16).all() and (ci < (b + 1) * R // 16).all()
    # same seed, same matrix; another seed, another one
    A2 = sel.gen_device(spec)
    assert np.array_equal(host(A2.d_rowPtr), rp) and np.array_equal(host(A2.d_colIdx)[:A.nnz], ci)
    assert np.array_equal(host(A2.d_values)[:A.nnz], host(A.d_values)[:A.nnz])
    spec.seed += 1
    A3 = sel.gen_device(spec)
    assert not np.array_equal(host(A3.d_rowPtr), rp) or not np.array_equal(host(A3.d_colIdx)[:A3.nnz], ci)


@pytest.mark.parametrize("kind", ["2d", "3d"])
def test_device_stencils_match_host_generator(mx, sel, cuda, kind):
    """Device stencil operators have the host generator's structure (and,
    for the 5-point Laplacian, its values)."""
    if kind == "2d":
        spec = mx.GenSpec(mx.GEN_STENCIL2D, 37 * 53, 37 * 53, 37.0, 53.0, 0.0, 0.0, 4)
    else:
        spec = mx.GenSpec(mx.GEN_STENCIL3D, 9 * 11 * 7, 9 * 11 * 7, 9.0, 11.0, 7.0, 0.0, 4)
    A = sel.gen_device(spec)
    cuda.cuda.synchronize()
    rp, ci, v = mx.generate(spec)
    assert np.array_equal(host(A.d_rowPtr), rp)
    assert np.array_equal(host(A.d_colIdx)[:A.nnz], ci)
    dv = host(A.d_values)[:A.nnz]
    if kind == "2d":
        assert np.array_equal(dv, v)
    else:
        assert abs(dv.astype(np.float64).mean()) < 0.1 and abs(dv.std() - 1.0) < 0.1


def test_device_generator_values_and_vector(mx, sel, cuda):
    _, A = _gen(mx, sel, mx.GEN_POISSON_UNIFORM, 20000, 30.0, 1.0, 80.0, seed=3)
    v = host(A.d_values)[:A.nnz].astype(np.float64)
    assert abs(v.mean()) < 0.02 and abs(v.std() - 1.0) < 0.02
    x = host(sel.gen_device_vector(100000, 9, -1.0, 1.0))
    assert x.min() >= -1.0 and x.max() <= 1.0 and abs(x.mean()) < 0.01
    assert np.array_equal(x, host(sel.gen_device_vector(100000, 9, -1.0, 1.0)))


# ---------------------------------------------------------------------------
# features
# ---------------------------------------------------------------------------
def features_ref(rp, ci, R, C, vsize, l2):
    """numpy restatement of the 32 selector features."""
    rp = rp.astype(np.int64)
    N = int(rp[-1])
    lens = np.diff(rp)
    Rd = max(R, 1)
    mean = lens.sum() / Rd
    var = (lens.astype(np.float64) ** 2).sum() / Rd - mean * mean
    sd = math.sqrt(var) if var > 0 else 0.0
    nn = max(N, 1)
    f = np.zeros(32)
    f[0], f[1], f[2], f[3] = math.log2(R + 1), math.log2(C + 1), math.log2(N + 1), math.log2(mean + 1)
    f[4] = sd / mean if mean > 0 else 0
    mx_ = int(lens.max()) if R else 0
    f[5] = math.log2(mx_ + 1)
    f[6] = math.log2((mx_ / mean if mean > 0 else 0) + 1)
    f[7] = (lens == 0).sum() / Rd
    edges = [0, 1, 2, 4, 8, 16, 32, 64, 128, 256, 1024, 4096]
    b = np.searchsorted(np.array(edges[1:]), lens, side="right")
    f[8:20] = np.bincount(b, minlength=12)[:12] / Rd
    f[20] = lens[lens >= 1024].sum() / nn
    f[21] = lens[lens >= 256].sum() / nn
    samples = min(R, 4096)
    dist = gap = 0.0
    n = n64 = n4k = nfr = pairs = close = 0
    span = 0.0
    spanRows = 0
    for w in range(samples):
        r = w if samples >= R else w * R // samples
        s, e0 = rp[r], rp[r + 1]
        e = min(e0, s + 1024)
        c = ci[s:e].astype(np.int64)
        if len(c) == 0:
            continue
        diag = r * C / max(R, 1)
        dd = np.abs(c - diag)
        dist += dd.sum()
        n += len(c)
        n64 += (dd <= 64).sum()
        n4k += (dd <= 4096).sum()
        nfr += (dd <= C / 64.0).sum()
        g = np.abs(np.diff(c))
        gap += g.sum()
        pairs += len(g)
        close += (g <= 8).sum()
        span += (c.max() - c.min()) / max(C, 1)
        spanRows += 1
    ns = max(n, 1)
    f[22] = dist / ns / max(C, 1)
    f[23], f[24], f[25] = n64 / ns, n4k / ns, nfr / ns
    f[26] = span / spanRows if spanRows else 0
    f[27] = math.log2((gap / pairs if pairs else 0) + 1)
    f[28] = close / pairs if pairs else 0
    f[29] = math.log2((C * vsize + 1) / l2)
    f[30] = math.log2((N * (vsize + 4) + (R + 1) * 4 + 1) / l2)
    f[31] = math.log2((R + 1) / (C + 1))
    return f


@pytest.mark.parametrize("case", ["poisson", "powerlaw", "banded_rect", "empties"])
def test_features_match_numpy(mx, sel, cuda, handle, case):
    from muxi_spmv_gb300 import workloads as W
    if case == "poisson":
        s = W.spec("poisson16k")
    elif case == "powerlaw":
        s = W.scaled("powerlaw8m", 50000, seed=1)
    elif case == "banded_rect":
        s = mx.GenSpec(mx.GEN_BANDED, 9000, 12000, 9.0, 33.0, 0.0, 0.0, 4)
    else:
        s = mx.GenSpec(mx.GEN_POISSON_UNIFORM, 5000, 700, 0.7, 0.0, 5.0, 0.0, 5)
    rp, ci, v = mx.generate(s)
    A = mx.CSRMatrix(rp, ci, v, s.numCols).copyToDevice()
    f = host(sel.matrix_features(A))
    ref = features_ref(rp, ci, A.numRows, A.numCols, 4, float(handle.l2CacheBytes))
    np.testing.assert_allclose(f, ref, rtol=2e-5, atol=1e-6)


# ---------------------------------------------------------------------------
# MLP
# ---------------------------------------------------------------------------
def _mlp_problem(cuda, shape, batch, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, (batch, shape[0])).astype(np.float32)
    T = rng.normal(0, 1, (batch, shape[3])).astype(np.float32)
    M = (rng.random((batch, shape[3])) < 0.7).astype(np.float32)
    mean = rng.normal(0, 0.2, shape[0]).astype(np.float32)
    std = rng.uniform(0.5, 2.0, shape[0]).astype(np.float32)
    d = [cuda.from_numpy(a).cuda() for a in (X, T, M)]
    return X, T, M, mean, std, d


@pytest.mark.parametrize("shape,batch", [((32, 128, 128, 24), 200), ((5, 7, 3, 4), 1), ((32, 17, 9, 24), 33)])
def test_mlp_forward_and_gradients_match_fp64(sel, cuda, shape, batch):
    X, T, M, mean, std, (dX, dT, dM) = _mlp_problem(cuda, shape, batch, 11)
    m = sel.MLP(*shape, seed=5)
    assert m.shape == shape and m.num_params == mlp_ref.num_params(shape)
    m.set_normalization(mean, std)
    p = m.get_params().astype(np.float64)
    Y = host(m.forward(dX)).astype(np.float64)
    Yr, _ = mlp_ref.forward(p, shape, mean.astype(np.float64), std.astype(np.float64), X.astype(np.float64))
    np.testing.assert_allclose(Y, Yr, rtol=1e-4, atol=1e-4 * np.abs(Yr).max())
    loss, g = m.gradients(dX, dT, dM)
    lr, gr = mlp_ref.loss_and_grads(p, shape, mean.astype(np.float64), std.astype(np.float64),
                                   X.astype(np.float64), T.astype(np.float64), M.astype(np.float64))
    assert loss == pytest.approx(lr, rel=1e-4)
    # FP32 kernels vs FP64: relative error of the whole gradient vector and per block
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)
    k = 0
    i, h1, h2, o = shape
    for size in (h1 * i, h1, h2 * h1, h2, o * h2, o):
        blk, ref = g[k:k + size], gr[k:k + size]
        assert np.linalg.norm(blk - ref) <= 1e-3 * max(np.linalg.norm(ref), 1e-6)
        k += size


def test_mlp_adam_matches_fp64(sel, cuda):
    shape, batch = (32, 64, 48, 24), 96
    X, T, M, mean, std, (dX, dT, dM) = _mlp_problem(cuda, shape, batch, 12)
    m = sel.MLP(*shape, seed=6)
    m.set_normalization(mean, std)
    mm = vv = None
    for step in range(1, 6):
        # The update is checked on the library's own gradient (its accuracy is
        # checked above), so the comparison isolates the Adam kernel.
        p = m.get_params().astype(np.float64)
        l_gpu, g = m.gradients(dX, dT, dM)
        g = g.astype(np.float64)
        if mm is None:
            mm, vv = np.zeros_like(p), np.zeros_like(p)
        p_ref, mm, vv = mlp_ref.adam(p, g, mm, vv, step, 1e-3)
        loss = m.train_step(dX, dT, dM, 1e-3, want_loss=True)
        assert loss == pytest.approx(l_gpu, rel=1e-6)
        np.testing.assert_allclose(m.get_params(), p_ref, rtol=0, atol=1e-6)


def test_mlp_training_reduces_loss(sel, cuda):
    """A learnable target (a fixed random 2-layer function of the inputs)."""
    rng = np.random.default_rng(3)
    X = rng.normal(0, 1, (512, 32)).astype(np.float32)
    W = rng.normal(0, 0.3, (32, 24))
    T = np.tanh(X @ W).astype(np.float32)
    M = np.ones_like(T)
    dX, dT, dM = (cuda.from_numpy(a).cuda() for a in (X, T, M))
    m = sel.MLP(32, 64, 64, 24, seed=1)
    l0, _ = m.gradients(dX, dT, dM)
    for _ in range(300):
        m.train_step(dX, dT, dM, 3e-3)
    l1, _ = m.gradients(dX, dT, dM)
    assert l1 < 0.1 * l0


def test_mlp_save_load_and_corruption(sel, cuda, tmp_path, mx):
    m = sel.MLP(32, 16, 8, 24, seed=9)
    m.set_normalization(np.arange(32, dtype=np.float32), np.full(32, 2.0, np.float32))
    path = tmp_path / "m.mxsmlp"
    m.save(path)
    m2 = sel.MLP.load(path)
    assert m2.shape == (32, 16, 8, 24)
    np.testing.assert_array_equal(m2.get_params(), m.get_params())
    X = cuda.randn(7, 32, device="cuda")
    assert cuda.equal(m.forward(X), m2.forward(X))
    b = bytearray(path.read_bytes())
    bad = tmp_path / "bad.mxsmlp"
    b[100] ^= 0x40
    bad.write_bytes(bytes(b))
    with pytest.raises(mx.SpmvError, match="checksum"):
        sel.MLP.load(bad)
    bad.write_bytes(path.read_bytes()[:-20])
    with pytest.raises(mx.SpmvError, match="truncated"):
        sel.MLP.load(bad)
    bad.write_bytes(b"NOTAMODEL" + path.read_bytes()[9:])
    with pytest.raises(mx.SpmvError, match="magic"):
        sel.MLP.load(bad)


# ---------------------------------------------------------------------------
# autotune / select / AUTO plans
# ---------------------------------------------------------------------------
def _small(mx, name):
    from muxi_spmv_gb300 import workloads as W
    s = W.spec("poisson16k") if name == "poisson" else W.scaled("powerlaw8m", 40000, seed=8)
    rp, ci, v = mx.generate(s)
    return rp, ci, v, mx.CSRMatrix(rp, ci, v, s.numCols).copyToDevice()


@pytest.mark.parametrize("name", ["poisson", "powerlaw"])
def test_autotune_reports_every_variant(mx, sel, cuda, handle, name):
    rp, ci, v, A = _small(mx, name)
    space = sel.variant_space()
    ms, best = sel.autotune(handle, A, None, repeats=0)
    assert len(ms) == len(space) == 28
    ok = ms > 0
    assert best == int(np.where(ok, ms, np.inf).argmin())
    maxlen = int(np.diff(rp).max())
    ell_ok = A.numRows * maxlen <= 2 * A.nnz
    ell = [i for i, v in enumerate(space) if v.kernel == mx.KERNEL_ELL]
    assert len(ell) == 1 and bool(ok[ell[0]]) == ell_ok
    assert all(ok[i] for i in range(len(space)) if i not in ell)


def test_select_modes(mx, sel, cuda, handle):
    rp, ci, v, A = _small(mx, "powerlaw")
    vh, ih = sel.select(handle, A, sel.SELECT_HEURISTIC)
    assert vh.kernel == mx.KERNEL_SCALAR and ih == 1  # mean row length < 32
    space = sel.variant_space()
    n = len(space)
    ell = next(i for i, v in enumerate(space) if v.kernel == mx.KERNEL_ELL)
    va, ia = sel.select(handle, A, sel.SELECT_AUTOTUNE)
    assert 0 <= ia < n
    model = sel.MLP(32, 32, 32, n, seed=2)
    vl, il = sel.select(handle, A, sel.SELECT_LEARNED, model)
    assert 0 <= il < n and space[il].as_dict() == vl.as_dict()
    assert il != ell  # ELL does not apply to this matrix
    f = sel.matrix_features(A).reshape(1, -1)
    pred = host(model.forward(f))[0]
    pred[ell] = np.inf
    assert il == int(pred.argmin())
    vk, ik = sel.select(handle, A, sel.SELECT_LEARNED_TOPK, model, topK=3)
    assert ik in list(np.argsort(pred, kind="stable")[:3])
    # fallback: the pick, or one of the variants predicted within the margin
    vf, iff = sel.select(handle, A, sel.SELECT_LEARNED_FALLBACK, model)
    near = [i for i in np.argsort(pred, kind="stable")[:sel.FALLBACK_MAX]
            if pred[i] - pred.min() <= sel.FALLBACK_MARGIN + 1e-6]
    assert iff in near and space[iff].as_dict() == vf.as_dict()
    with pytest.raises(mx.SpmvError):
        sel.select(handle, A, sel.SELECT_LEARNED, None)
    with pytest.raises(mx.SpmvError):
        sel.set_selector(handle, sel.MLP(32, 8, 8, 5))


def test_auto_plan_with_registered_selector(mx, sel, cuda):
    h = mx.spmv_create_handle()
    rp, ci, v, A = _small(mx, "powerlaw")
    model = sel.MLP(32, 32, 32, len(sel.variant_space()), seed=4)
    sel.set_selector(h, model)
    vl, il = sel.select(h, A, sel.SELECT_LEARNED, model)
    plan = mx.Plan(h, A)
    pv = plan.variant
    assert (pv.kernel, pv.blockSize, pv.threadsPerRow, pv.itemsPerThread) == \
        (vl.kernel, vl.blockSize, vl.threadsPerRow, vl.itemsPerThread)
    x = mx.gen_vector(A.numCols, 5)
    y = cuda.zeros(A.numRows, device="cuda")
    plan.exec(cuda.from_numpy(x).cuda(), y)
    y_ref, absum = oracle.spmv_ref(rp, ci, v, x)
    assert oracle.row_errors(host(y), y_ref, absum, tol_for(np.float32)).max() <= 1.0
    # fallback mode: the plan's variant is one of those predicted within the margin
    sel.set_selector(h, model, sel.SELECT_LEARNED_FALLBACK)
    pred = host(model.forward(sel.matrix_features(A).reshape(1, -1)))[0]
    space = sel.variant_space()
    plan2 = mx.Plan(h, A)
    key = lambda v: (v.kernel, v.blockSize, v.threadsPerRow, v.itemsPerThread, v.vectorWidth)
    near = [key(space[i]) for i in np.argsort(pred, kind="stable")[:sel.FALLBACK_MAX]
            if pred[i] - pred[il] <= sel.FALLBACK_MARGIN + 1e-6]
    assert key(plan2.variant) in near or key(plan2.variant) == key(vl)
    y2 = cuda.zeros(A.numRows, device="cuda")
    plan2.exec(cuda.from_numpy(x).cuda(), y2)
    assert oracle.row_errors(host(y2), y_ref, absum, tol_for(np.float32)).max() <= 1.0
    with pytest.raises(mx.SpmvError):  # AUTO plans take the learned modes only
        mx.check(mx.lib().spmv_set_selector_mode(h.raw, sel.SELECT_AUTOTUNE), "spmv_set_selector_mode")
    # FP64 AUTO plans keep the FP64 default whatever the model says (its labels are FP32 timings)
    A64 = device_csr(mx, rp, ci, v.astype(np.float64), A.numCols)
    for mode in (sel.SELECT_LEARNED, sel.SELECT_LEARNED_FALLBACK):
        sel.set_selector(h, model, mode)
        pv64 = mx.Plan(h, A64).variant
        assert (pv64.kernel, pv64.blockSize, pv64.itemsPerThread, pv64.vectorWidth) == (mx.KERNEL_CSR5, 128, 8, 32)
    sel.set_selector(h, None)
    assert mx.Plan(h, A).variant.kernel == mx.KERNEL_CSR5
    h.destroy()


DEFAULT_MODEL = Path(__file__).resolve().parents[1] / "muxi_spmv_gb300" / "data" / "selector_gb300.mxsmlp"


@pytest.mark.skipif(not DEFAULT_MODEL.exists(), reason="no trained selector model committed")
def test_committed_model_selects_and_matches_oracle(mx, sel, cuda, handle):
    model = sel.MLP.load(DEFAULT_MODEL)
    assert model.shape == (32, 128, 128, len(sel.variant_space()))
    for name in ("poisson", "powerlaw"):
        rp, ci, v, A = _small(mx, name)
        vl, il = sel.select(handle, A, sel.SELECT_LEARNED, model)
        plan = mx.Plan(handle, A, vl)
        x = mx.gen_vector(A.numCols, 6)
        y = cuda.zeros(A.numRows, device="cuda")
        plan.exec(cuda.from_numpy(x).cuda(), y)
        y_ref, absum = oracle.spmv_ref(rp, ci, v, x)
        assert oracle.row_errors(host(y), y_ref, absum, tol_for(np.float32)).max() <= 1.0


@pytest.mark.skipif(not DEFAULT_MODEL.exists(), reason="no trained selector model committed")
def test_committed_model_on_held_out_corpus_gpu(sel, cuda):
    """The CUDA forward pass on the committed held-out records: learned
    regret <= 5% and below the reference heuristic and the fixed default."""
    from muxi_spmv_gb300 import selector_train as st
    corpus = DEFAULT_MODEL.parent / "selector_corpus_gb300.npz"
    d = dict(np.load(corpus))
    model = sel.MLP.load(DEFAULT_MODEL)
    rep = st.evaluate(model, d, "test")
    assert rep["learned_regret"]["mean"] <= 0.05
    assert rep["learned_regret"]["mean"] < rep["heuristic_regret"]["mean"]
    assert rep["learned_regret"]["mean"] < rep["default_csr5_regret"]["mean"]


@pytest.mark.skipif(not DEFAULT_MODEL.exists(), reason="no trained selector model committed")
def test_learned_selection_is_100x_cheaper_than_autotune(mx, sel, cuda, handle):
    """The selection-cost claim, re-measured: on three corpus matrices of
    different laws (banded rows, a grid stencil, power-law rows), the learned
    pick (features + MLP forward + rank, median of 10 warm calls) costs at
    least 100x less wall time than the exhaustive autotune the corpus labels
    come from (spmv_autotune over the whole space, every variant built as a
    plan and timed for about 2 ms)."""
    import time
    from muxi_spmv_gb300 import selector_train as st
    model = sel.MLP.load(DEFAULT_MODEL)
    ratios = []
    for seed in (6, 1_000_002, 2_000_003):  # banded, stencil, power law
        spec, law, _ = st.spec_for_seed(seed, max_rows=1_000_000)
        if law == "powerlaw":
            rp, ci, v = mx.generate(spec)
            A = mx.CSRMatrix(rp, ci, v, spec.numCols).copyToDevice()
        else:
            A = sel.gen_device(spec)
        cuda.cuda.synchronize()
        sel.select(handle, A, sel.SELECT_LEARNED, model)  # warm
        t = []
        for _ in range(10):
            cuda.cuda.synchronize()
            t0 = time.perf_counter()
            sel.select(handle, A, sel.SELECT_LEARNED, model)
            cuda.cuda.synchronize()
            t.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        sel.autotune(handle, A, None, repeats=0)
        cuda.cuda.synchronize()
        ratios.append((time.perf_counter() - t0) / float(np.median(t)))
    assert min(ratios) >= 100.0, ratios
