"""Selector host-side checks that need no GPU: the FP64 restatement of the
MLP against finite differences, the corpus law sampler, the model file
format, and selection quality of the committed model on the committed
held-out corpus records."""
import math
import struct
from pathlib import Path

import numpy as np
import pytest

import mlp_ref
from muxi_spmv_gb300 import selector_train as st

DATA = Path(__file__).resolve().parents[1] / "muxi_spmv_gb300" / "data"
MODEL = DATA / "selector_gb300.mxsmlp"
CORPUS = DATA / "selector_corpus_gb300.npz"


def _problem(shape, batch, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, mlp_ref.num_params(shape))
    X = rng.normal(0, 1, (batch, shape[0]))
    T = rng.normal(0, 1, (batch, shape[3]))
    M = (rng.random((batch, shape[3])) < 0.7).astype(np.float64)
    mean = rng.normal(0, 0.1, shape[0])
    std = rng.uniform(0.5, 2.0, shape[0])
    return p, X, T, M, mean, std


def test_numpy_mlp_gradients_match_finite_differences():
    shape = (6, 5, 4, 3)
    p, X, T, M, mean, std = _problem(shape, 9)
    loss, g = mlp_ref.loss_and_grads(p, shape, mean, std, X, T, M)
    assert math.isclose(loss, mlp_ref.loss_only(p, shape, mean, std, X, T, M), rel_tol=1e-12)
    eps = 1e-6
    fd = np.empty_like(p)
    for i in range(p.size):
        a, b = p.copy(), p.copy()
        a[i] += eps
        b[i] -= eps
        fd[i] = (mlp_ref.loss_only(a, shape, mean, std, X, T, M) - mlp_ref.loss_only(b, shape, mean, std, X, T, M)) / (2 * eps)
    np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-8)


def test_numpy_adam_first_step_moves_by_lr():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -4.0, 0.0])
    p2, m, v = mlp_ref.adam(p, g, np.zeros(3), np.zeros(3), 1, 0.01)
    # first bias-corrected step is lr * sign(g) (eps aside)
    np.testing.assert_allclose(p2, p - 0.01 * np.sign(g), atol=1e-7)


def test_corpus_specs_are_deterministic_and_in_range():
    for seed in range(40):
        s1, law1, m1 = st.spec_for_seed(seed)
        s2, law2, m2 = st.spec_for_seed(seed)
        assert s1 == s2 and law1 == law2 and m1 == m2
        assert 10_000 <= s1.numRows <= 10_000_000
        assert 2.0 <= m1 <= 128.0
        assert law1 == st.LAWS[seed % 4]
        if law1 == "zipf":
            assert 1.3 <= s1.p0 <= 2.5 and s1.p1 >= 1
        if law1 == "banded":
            assert 3 <= s1.p1 <= 1025
        if law1 == "blockdiag":
            assert 8 <= s1.p0 <= 256


def test_zipf_clip_gives_requested_mean():
    for s, target in ((1.3, 50.0), (1.8, 8.0), (2.2, 1.5)):
        K = st._zipf_clip_for_mean(s, target, 1 << 20)
        k = np.arange(1, K + 1, dtype=np.float64)
        mean = (k ** (1 - s)).sum() / (k ** -s).sum()
        assert mean <= target + 1e-9
        k2 = np.arange(1, K + 2, dtype=np.float64)
        if K < (1 << 20):
            assert (k2 ** (1 - s)).sum() / (k2 ** -s).sum() > target


def test_targets_and_regret_helpers():
    ms = np.array([[2.0, 1.0, -1.0, 4.0], [1.0, 3.0, 2.0, 100.0]])
    T, M = st.targets(ms)
    np.testing.assert_array_equal(M, [[1, 1, 0, 1], [1, 1, 1, 1]])
    np.testing.assert_allclose(T[0], [math.log(2), 0, 0, math.log(4)], rtol=1e-6)
    assert T[1, 3] == pytest.approx(math.log(20.0))  # clipped
    r = st.regrets(np.array([0, 0]), ms)
    np.testing.assert_allclose(r, [1.0, 0.0])
    picks = st.learned_picks(np.array([[0.0, 1.0, -5.0, 2.0], [3.0, 2.0, 1.0, 0.0]]), ms)
    np.testing.assert_array_equal(picks, [0, 3])  # the inapplicable variant is never picked


def _parse_model(path):
    b = path.read_bytes()
    assert b[:8] == b"MXSMLP01"
    ver, i, h1, h2, o = struct.unpack("<5i", b[8:28])
    n = mlp_ref.num_params((i, h1, h2, o))
    need = 28 + 4 * (n + 2 * i) + 8
    assert len(b) == need
    # FNV-1a 64 over everything before the trailing checksum
    h = 1469598103934665603
    for c in b[:-8]:
        h ^= c
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    assert struct.unpack("<Q", b[-8:])[0] == h
    f = np.frombuffer(b[28:-8], np.float32)
    return ver, (i, h1, h2, o), f[:n].astype(np.float64), f[n:n + i].astype(np.float64), f[n + i:].astype(np.float64)


@pytest.mark.skipif(not MODEL.exists(), reason="no trained selector model committed")
def test_committed_model_file_is_well_formed():
    ver, shape, p, mean, std = _parse_model(MODEL)
    assert ver == 1 and shape[0] == 32 and shape[1] == 128 and shape[2] == 128
    assert np.isfinite(p).all() and (std > 0).all()


@pytest.mark.skipif(not (MODEL.exists() and CORPUS.exists()), reason="no trained selector committed")
def test_committed_model_beats_non_learned_selection_on_held_out_seeds():
    """Regret on held-out corpus seeds (seed % 5 == 0), FP64 restatement of
    the forward pass: learned mean regret <= 5% and below both the
    reference's heuristic rule and the fixed CSR5 default."""
    _, shape, p, mean, std = _parse_model(MODEL)
    d = np.load(CORPUS)
    meta, ms_all, X = d["meta"], d["ms"], d["features"]
    te = (meta[:, 0].astype(np.int64) % 5) == 0
    assert te.sum() >= 100
    ms = ms_all[te, :-1]
    pred, _ = mlp_ref.forward(p, shape, mean, std, X[te])
    picks = st.learned_picks(pred, ms)
    r_learn = st.regrets(picks, ms)
    r_heur = st.regrets(None, ms, ms_pick=ms_all[te, -1])
    r_def = st.regrets(np.full(te.sum(), st.default_index()), ms)
    assert r_learn.mean() <= 0.05
    assert r_learn.mean() < r_heur.mean()
    assert r_learn.mean() < r_def.mean()
    # the low-confidence fallback (time the variants predicted within 12% of
    # the pick, at most 4) only helps, and times fewer than its cap on average
    r_fb, n_fb = st.fallback_regrets(pred, ms)
    assert (r_fb <= r_learn + 1e-12).all()
    assert r_fb.mean() < r_learn.mean() and np.percentile(r_fb, 95) < np.percentile(r_learn, 95)
    assert 1.0 <= n_fb.mean() < st.selector.FALLBACK_MAX
