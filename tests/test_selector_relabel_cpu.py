"""The corpus relabel command (selector_train relabel) on the host: records
are re-timed for one variant only, in resumable chunks, and merged into that
column alone; a regenerated matrix whose shape differs from its record stops
the run.  The generator and the timer are replaced by fakes, so no GPU is
involved."""
from __future__ import annotations

import argparse
import types

import numpy as np
import pytest

from muxi_spmv_gb300 import selector_train as st


def _corpus(n=7, cols=29):
    meta = np.zeros((n, 7))
    meta[:, 0] = np.arange(100, 100 + n)  # seeds
    meta[:, 2] = 1000 + np.arange(n)      # rows
    meta[:, 3] = 1000 + np.arange(n)      # columns
    meta[:, 4] = 5000 + np.arange(n)      # nonzeros
    ms = np.arange(n * cols, dtype=np.float32).reshape(n, cols) + 1.0
    return {"features": np.zeros((n, 32), np.float32), "ms": ms, "meta": meta}


@pytest.fixture
def fakes(monkeypatch):
    calls = []

    def corpus_matrix(seed, max_rows, max_nnz):
        i = seed - 100
        A = types.SimpleNamespace(numRows=1000 + i, numCols=1000 + i, nnz=5000 + i)
        if seed == fakes.bad_seed:
            A.nnz += 1
        return A, "poisson", 5.0

    def autotune(handle, A, cands, repeats=0):
        calls.append((A.numRows, len(cands)))
        return np.array([0.5 + A.numRows / 1e4], np.float32), 0

    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(init=lambda: None, empty_cache=lambda: None))
    monkeypatch.setitem(__import__("sys").modules, "torch", fake_torch)
    monkeypatch.setattr(st, "corpus_matrix", corpus_matrix)
    monkeypatch.setattr(st.selector, "autotune", autotune)
    monkeypatch.setattr(st.selector, "variant_space", lambda: list(range(28)))
    monkeypatch.setattr(st.api, "SpmvHandle", lambda: object())
    fakes.bad_seed = -1
    fakes.calls = calls
    return fakes


def _args(tmp_path, corpus, **kw):
    a = dict(corpus=str(corpus), index=21, out=str(tmp_path / "chunks"), merged=str(tmp_path / "merged.npz"),
             chunk=3, max_rows=10_000_000, max_nnz=600_000_000, time_limit=0.0)
    a.update(kw)
    return argparse.Namespace(**a)


def test_relabel_replaces_one_column(tmp_path, fakes):
    data = _corpus()
    path = tmp_path / "corpus.npz"
    st.save_corpus(data, path)
    st.cmd_relabel(_args(tmp_path, path))
    out = np.load(tmp_path / "merged.npz")
    want = data["ms"].copy()
    want[:, 21] = 0.5 + data["meta"][:, 2] / 1e4
    np.testing.assert_allclose(out["ms"], want, rtol=1e-6)
    np.testing.assert_array_equal(out["meta"], data["meta"])
    assert len(fakes.calls) == 7 and all(k == 1 for _, k in fakes.calls)  # one variant timed per record
    assert sorted(p.name for p in (tmp_path / "chunks").iterdir()) == [
        "relabel_21_000000.npy", "relabel_21_000003.npy", "relabel_21_000006.npy"]


def test_relabel_resumes_from_finished_chunks(tmp_path, fakes):
    path = tmp_path / "corpus.npz"
    st.save_corpus(_corpus(), path)
    (tmp_path / "chunks").mkdir()
    np.save(tmp_path / "chunks" / "relabel_21_000000.npy", np.full(3, 9.0, np.float32))
    st.cmd_relabel(_args(tmp_path, path))
    out = np.load(tmp_path / "merged.npz")
    np.testing.assert_array_equal(out["ms"][:3, 21], 9.0)  # the finished chunk is kept, not re-timed
    assert len(fakes.calls) == 4


def test_relabel_stops_on_a_shape_mismatch(tmp_path, fakes):
    path = tmp_path / "corpus.npz"
    st.save_corpus(_corpus(), path)
    fakes.bad_seed = 104
    with pytest.raises(SystemExit, match="seed 104"):
        st.cmd_relabel(_args(tmp_path, path))
    assert not (tmp_path / "merged.npz").exists()


def test_relabel_rejects_an_index_outside_the_space(tmp_path, fakes):
    path = tmp_path / "corpus.npz"
    st.save_corpus(_corpus(), path)
    with pytest.raises(SystemExit, match="outside the variant space"):
        st.cmd_relabel(_args(tmp_path, path, index=28))
