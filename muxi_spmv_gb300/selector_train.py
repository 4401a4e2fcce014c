"""Builds the learned kernel selector: corpus, training, evaluation.

    python -m muxi_spmv_gb300.selector_train corpus --out DIR [--count 4000]
    python -m muxi_spmv_gb300.selector_train train --corpus DIR --model OUT.mxsmlp
    python -m muxi_spmv_gb300.selector_train evaluate --corpus DIR --model OUT.mxsmlp

corpus: seeded matrices generated on the GPU, one law per seed -- Poisson row
lengths, Zipf lengths (s in [1.3, 2.5]), banded (width 3..1025) and
block-diagonal (8..256 blocks) -- with rows log-uniform in [1e4, 1e7] and mean
row length log-uniform in [2, 128], FP32 N(0,1) values; seeds from
STENCIL_SEED0 on are grid stencils (2D 5-point, 3D 27-point; from
LARGE_STENCIL_SEED0 on at the benchmark's 1e7-row scale), from
POWERLAW_SEED0 on power-law rows with a near-diagonal share (from
LARGE_POWERLAW_SEED0 on with 2e6..1e7 rows).  Each matrix gets its
32 features (spmv_matrix_features) and the exhaustive autotuner's time for
every variant of the space plus the reference heuristic's pick.  Records are
written in chunks, so an interrupted run resumes where it stopped.

train: targets are log(time / best time) per variant, masked where a variant
does not apply; seeds with seed % 5 == 0 are held out (80/20 split by seed).
The network (32 -> 128 -> 128 -> variants) is trained on the GPU by the
library's own kernels (spmv_mlp_train_step).

evaluate: regret = time of the pick / best time - 1 on the held-out seeds,
for the learned selector, the reference heuristic (src/spmv/csr/spmv_csr.cu:
115-153) and the fixed default (CSR5, 256-nonzero tiles); selection cost =
wall time of spmv_select(LEARNED) against the autotuner's wall time.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

from . import api, selector
from .api import (GenSpec, GEN_BANDED, GEN_BLOCKDIAG, GEN_POISSON_UNIFORM, GEN_POWERLAW, GEN_STENCIL2D,
                  GEN_STENCIL3D, GEN_ZIPF_UNIFORM, Variant)

LAWS = ("poisson", "zipf", "banded", "blockdiag", "stencil", "powerlaw")
# Seeds from STENCIL_SEED0 draw grid stencils (2D 5-point or 3D 27-point),
# from POWERLAW_SEED0 power-law rows with a near-diagonal share (the
# benchmark's law, generated on the host); below both the law is
# LAWS[seed % 4].
STENCIL_SEED0 = 1_000_000
LARGE_STENCIL_SEED0 = 1_000_500  # after the 500 stencil seeds of the first range
POWERLAW_SEED0 = 2_000_000
LARGE_POWERLAW_SEED0 = 2_000_250  # after the 250 power-law seeds of up to 2e6 rows
HEURISTIC_COL = -1  # last column of the label matrix: the heuristic's variant
DEFAULT_VARIANT = Variant(api.KERNEL_CSR5, 128, 0, 16, 32)  # the FP32 AUTO plan without a model


def _zipf_clip_for_mean(s: float, target: float, cap: int) -> int:
    """Largest truncation K <= cap whose Zipf(s) mean is <= target (at least 1)."""
    K = np.arange(1, cap + 1, dtype=np.float64)
    w = K ** (-s)
    mean = np.cumsum(w * K) / np.cumsum(w)
    k = int(np.searchsorted(mean, target, side="right"))
    return max(1, min(cap, k))


def spec_for_seed(seed: int, max_rows: int = 10_000_000, max_nnz: int = 600_000_000):
    """The corpus matrix of `seed`: (GenSpec, law name, target mean row length)."""
    rng = np.random.default_rng(np.random.SeedSequence([0x5E1EC7, seed]))
    if seed >= POWERLAW_SEED0:
        return powerlaw_spec(rng, seed, max_rows)
    if seed >= STENCIL_SEED0:
        return stencil_spec(rng, seed, max_rows)
    law = LAWS[seed % 4] if seed >= 0 else LAWS[0]
    lo = math.log10(1e4)
    R = int(round(10 ** rng.uniform(lo, math.log10(max_rows))))
    m = float(10 ** rng.uniform(math.log10(2.0), math.log10(128.0)))
    if R * m > max_nnz:
        R = max(10_000, int(max_nnz / m))
    C = R
    gseed = 1_000_003 * seed + 17
    if law == "poisson":
        spec = GenSpec(GEN_POISSON_UNIFORM, R, C, m, 0.0, float(min(C, int(4 * m + 64))), 0.0, gseed)
    elif law == "zipf":
        s = float(rng.uniform(1.3, 2.5))
        clip = _zipf_clip_for_mean(s, m, min(C, 1 << 20))
        spec = GenSpec(GEN_ZIPF_UNIFORM, R, C, s, float(clip), 0.0, 0.0, gseed)
    elif law == "banded":
        w = int(round(10 ** rng.uniform(math.log10(3), math.log10(1025))))
        w = max(3, min(w, C))
        spec = GenSpec(GEN_BANDED, R, C, min(m, float(w)), float(w), 0.0, 0.0, gseed)
    else:
        nb = int(rng.integers(8, 257))
        spec = GenSpec(GEN_BLOCKDIAG, R, C, float(nb), m, 0.0, 0.0, gseed)
    return spec, law, m


def stencil_spec(rng, seed: int, max_rows: int):
    """A 2D 5-point grid (rows log-uniform 1e4..max_rows, aspect 1..16) or a
    3D 27-point grid (rows log-uniform 1e4..max_rows/4); from
    LARGE_STENCIL_SEED0 on, 2D grids of 1e7..2e7 rows and 3D grids of
    2.5e6..1.7e7 rows (the benchmark's 16.8M-row stencils)."""
    gseed = 1_000_003 * seed + 17
    large = seed >= LARGE_STENCIL_SEED0
    lo2, hi2 = (7.0, math.log10(2e7)) if large else (4.0, math.log10(max_rows))
    lo3, hi3 = (math.log10(2.5e6), math.log10(1.7e7)) if large else (4.0, math.log10(max_rows / 4))
    if rng.uniform() < 0.5:
        R = 10 ** rng.uniform(lo2, hi2)
        aspect = 2 ** rng.uniform(0, 4)
        ny = max(2, int(round(math.sqrt(R * aspect))))
        nx = max(2, int(round(R / ny)))
        spec = GenSpec(GEN_STENCIL2D, nx * ny, nx * ny, float(nx), float(ny), 0.0, 0.0, gseed)
        return spec, "stencil", 5.0
    R = 10 ** rng.uniform(lo3, hi3)
    dims = [max(2, int(round(R ** (1 / 3) * 2 ** rng.uniform(-0.5, 0.5)))) for _ in range(2)]
    n0 = max(2, int(round(R / (dims[0] * dims[1]))))
    n = n0 * dims[0] * dims[1]
    spec = GenSpec(GEN_STENCIL3D, n, n, float(n0), float(dims[0]), float(dims[1]), 0.0, gseed)
    return spec, "stencil", 27.0


def powerlaw_spec(rng, seed: int, max_rows: int):
    """Zipf(s) row lengths, s in [1.5, 2.2], clipped at 256..65,536; a share
    p in [0.3, 0.95] of the columns within +-band (band 64..8,192) of the
    diagonal, the rest uniform; rows log-uniform 1e4..min(max_rows, 2e6), and
    from LARGE_POWERLAW_SEED0 on log-uniform 2e6..min(max_rows, 1e7) (the
    benchmark's 8.4M-row scale, where other kernels win than at 2e6 rows)."""
    gseed = 1_000_003 * seed + 17
    if seed >= LARGE_POWERLAW_SEED0:
        R = int(round(10 ** rng.uniform(math.log10(2_000_000), math.log10(min(max_rows, 10_000_000)))))
    else:
        R = int(round(10 ** rng.uniform(4, math.log10(min(max_rows, 2_000_000)))))
    s = float(rng.uniform(1.5, 2.2))
    clip = int(2 ** rng.integers(8, 17))
    band = int(round(2 ** rng.uniform(6, 13)))
    p = float(rng.uniform(0.3, 0.95))
    spec = GenSpec(GEN_POWERLAW, R, R, s, float(min(clip, R)), float(min(band, R // 2)), p, gseed)
    return spec, "powerlaw", 0.0


def default_index() -> int:
    """Index in the variant space of the AUTO plan's variant without a model."""
    key = lambda v: (v.kernel, v.blockSize, v.threadsPerRow, v.itemsPerThread, v.vectorWidth)
    return next(i for i, v in enumerate(selector.variant_space()) if key(v) == key(DEFAULT_VARIANT))


def heuristic_variant(R: int, N: int) -> Variant:
    """The reference's dispatch rule (src/spmv/csr/spmv_csr.cu:115-153)."""
    avg = N // max(R, 1)
    if avg < 32:
        return Variant(api.KERNEL_SCALAR, 256, 1, 0, 1)
    return Variant(api.KERNEL_VECTOR, 256, 32, 0, 1)


def corpus_matrix(seed: int, max_rows: int, max_nnz: int):
    """The corpus matrix of `seed` on the device: (matrix, law, mean row length)."""
    import torch
    spec, law, m = spec_for_seed(seed, max_rows, max_nnz)
    if law == "powerlaw":  # no device law: host generator, copied over
        rp, ci, v = api.generate(spec)
        A = selector.DeviceCSR(spec.numRows, spec.numCols, len(ci), torch.from_numpy(rp).cuda(),
                               torch.from_numpy(ci if len(ci) else np.zeros(1, np.int32)).cuda(),
                               torch.from_numpy(v if len(v) else np.zeros(1, np.float32)).cuda())
        m = len(ci) / max(spec.numRows, 1)
    else:
        A = selector.gen_device(spec)
    torch.cuda.synchronize()
    return A, law, m


def label_one(handle, seed: int, max_rows: int, max_nnz: int):
    """Generates, featurises and autotunes one corpus matrix."""
    import torch
    A, law, m = corpus_matrix(seed, max_rows, max_nnz)
    feats = selector.matrix_features(A).cpu().numpy()
    space = selector.variant_space()
    cands = space + [heuristic_variant(A.numRows, A.nnz)]
    t0 = time.perf_counter()
    ms, _ = selector.autotune(handle, A, cands, repeats=0)
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t0
    meta = np.array([seed, LAWS.index(law), A.numRows, A.numCols, A.nnz, m, tune_s], np.float64)
    del A
    return feats, ms, meta


def cmd_corpus(a):
    import torch
    out = Path(a.out)
    out.mkdir(parents=True, exist_ok=True)
    handle = api.SpmvHandle()
    torch.cuda.init()
    t_start = time.perf_counter()
    for c0 in range(a.start, a.start + a.count, a.chunk):
        path = out / f"corpus_{c0:06d}.npz"
        if path.exists():
            continue
        F, L, Mt = [], [], []
        for seed in range(c0, min(c0 + a.chunk, a.start + a.count)):
            f, ms, meta = label_one(handle, seed, a.max_rows, a.max_nnz)
            F.append(f)
            L.append(ms)
            Mt.append(meta)
            torch.cuda.empty_cache()
        tmp = out / f".corpus_{c0:06d}.tmp.npz"
        np.savez(tmp, features=np.stack(F), ms=np.stack(L), meta=np.stack(Mt))
        tmp.rename(path)
        el = time.perf_counter() - t_start
        print(f"chunk {c0}: {len(F)} matrices, {el:.0f}s elapsed", flush=True)
        if a.time_limit and el > a.time_limit:
            print("time limit reached; rerun to resume", flush=True)
            break


def cmd_relabel(a):
    """Re-times one variant of the space (index a.index) on every record of
    a corpus, regenerating each matrix from its seed (its rows, columns and
    nonzeros must match the record), in resumable chunks under a.out; once
    every chunk is there, writes the corpus with that column replaced to
    a.merged."""
    import torch
    data = load_corpus(a.corpus)
    meta = data["meta"]
    space = selector.variant_space()
    if not 0 <= a.index < len(space):
        raise SystemExit(f"index {a.index} outside the variant space of {len(space)}")
    v = space[a.index]
    out = Path(a.out)
    out.mkdir(parents=True, exist_ok=True)
    handle = api.SpmvHandle()
    torch.cuda.init()
    t_start = time.perf_counter()
    n = len(meta)
    for c0 in range(0, n, a.chunk):
        path = out / f"relabel_{a.index:02d}_{c0:06d}.npy"
        if path.exists():
            continue
        col = []
        for i in range(c0, min(c0 + a.chunk, n)):
            A, _, _ = corpus_matrix(int(meta[i, 0]), a.max_rows, a.max_nnz)
            if (A.numRows, A.numCols, A.nnz) != tuple(int(z) for z in meta[i, 2:5]):
                raise SystemExit(f"seed {int(meta[i, 0])}: regenerated shape differs from the record")
            ms, _ = selector.autotune(handle, A, [v], repeats=0)
            col.append(float(ms[0]))
            del A
            torch.cuda.empty_cache()
        tmp = out / f".relabel_{a.index:02d}_{c0:06d}.tmp.npy"
        np.save(tmp, np.array(col, np.float32))
        tmp.rename(path)
        el = time.perf_counter() - t_start
        print(f"chunk {c0}: {len(col)} matrices, {el:.0f}s elapsed", flush=True)
        if a.time_limit and el > a.time_limit:
            print("time limit reached; rerun to resume", flush=True)
            return
    parts = [np.load(out / f"relabel_{a.index:02d}_{c0:06d}.npy") for c0 in range(0, n, a.chunk)]
    data = dict(data)
    data["ms"] = data["ms"].copy()
    data["ms"][:, a.index] = np.concatenate(parts)
    save_corpus(data, a.merged)
    print(f"wrote {a.merged}", flush=True)


def load_corpus(spec: str) -> dict:
    """Records of one or more corpora (comma-separated): chunk directories
    written by `corpus`, or merged .npz files (save_corpus)."""
    files = []
    for d in str(spec).split(","):
        p = Path(d)
        files += [p] if p.is_file() else sorted(p.glob("corpus_*.npz"))
    if not files:
        raise FileNotFoundError(f"no corpus records in {spec}")
    parts = [np.load(f) for f in files]
    return {k: np.concatenate([p[k] for p in parts]) for k in ("features", "ms", "meta")}


def save_corpus(data: dict, path) -> None:
    np.savez_compressed(path, **{k: data[k] for k in ("features", "ms", "meta")})


def targets(ms_space: np.ndarray, clip: float = math.log(20.0)):
    """log slowdown vs the best applicable variant, and the applicability mask."""
    M = (ms_space > 0).astype(np.float32)
    best = np.where(M > 0, ms_space, np.inf).min(1, keepdims=True)
    T = np.where(M > 0, np.log(np.maximum(ms_space, 1e-9) / best), 0.0)
    return np.minimum(T, clip).astype(np.float32), M


def split(meta: np.ndarray):
    test = (meta[:, 0].astype(np.int64) % 5) == 0
    return ~test, test


def regrets(pred_or_pick, ms_space: np.ndarray, ms_pick=None):
    """Per-matrix regret of a pick: picks index the space, or ms_pick gives times."""
    valid = ms_space > 0
    best = np.where(valid, ms_space, np.inf).min(1)
    if ms_pick is None:
        pick = pred_or_pick
        t = ms_space[np.arange(len(pick)), pick]
    else:
        t = ms_pick
    return t / best - 1.0


def learned_picks(pred: np.ndarray, ms_space: np.ndarray):
    return np.where(ms_space > 0, pred, np.inf).argmin(1)


def fallback_regrets(pred: np.ndarray, ms_space: np.ndarray, margin: float = selector.FALLBACK_MARGIN,
                     kmax: int = selector.FALLBACK_MAX):
    """SELECT_LEARNED_FALLBACK on recorded times: the learned pick plus the
    variants predicted within `margin` of it (at most kmax), fastest of them.
    Returns (regret per matrix, candidates timed per matrix)."""
    p = np.where(ms_space > 0, pred, np.inf)
    order = np.argsort(p, 1, kind="stable")
    best = np.where(ms_space > 0, ms_space, np.inf).min(1)
    reg, cnt = np.empty(len(p)), np.empty(len(p), np.int64)
    for r in range(len(p)):
        o = order[r]
        k = 1
        while k < kmax and np.isfinite(p[r, o[k]]) and p[r, o[k]] - p[r, o[0]] <= margin:
            k += 1
        reg[r] = ms_space[r, o[:k]].min() / best[r] - 1.0
        cnt[r] = k
    return reg, cnt


def cmd_train(a):
    import torch
    data = load_corpus(a.corpus)
    ms = data["ms"][:, :HEURISTIC_COL]
    tr, te = split(data["meta"])
    X = data["features"].astype(np.float32)
    T, M = targets(ms)
    mean = X[tr].mean(0)
    std = X[tr].std(0)
    nvar = ms.shape[1]
    model = selector.MLP(X.shape[1], a.hidden, a.hidden, nvar, seed=a.seed)
    model.set_normalization(mean, np.where(std > 1e-6, std, 1.0))
    dev = torch.device("cuda")
    Xtr, Ttr, Mtr = (torch.from_numpy(v[tr]).to(dev).contiguous() for v in (X, T, M))
    n = Xtr.shape[0]
    g = torch.Generator(device="cpu").manual_seed(a.seed)
    t0 = time.perf_counter()
    step = 0
    for ep in range(a.epochs):
        perm = torch.randperm(n, generator=g).to(dev)
        lr = a.lr * 0.5 * (1 + math.cos(math.pi * ep / a.epochs))
        for i in range(0, n, a.batch):
            idx = perm[i:i + a.batch]
            model.train_step(Xtr[idx].contiguous(), Ttr[idx].contiguous(), Mtr[idx].contiguous(), lr)
            step += 1
        if (ep + 1) % max(1, a.epochs // 10) == 0:
            loss, _ = model.gradients(Xtr, Ttr, Mtr)
            print(f"epoch {ep + 1}: train loss {loss:.4f}", flush=True)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    model.save(a.model)
    if a.merged:
        save_corpus(data, a.merged)
    rep = evaluate(model, data)
    rep["by_law"] = evaluate_by_law(model, data)
    rep["train_seconds"] = train_s
    rep["train_steps"] = step
    print(json.dumps(rep, indent=1))
    if a.report:
        Path(a.report).write_text(json.dumps(rep, indent=1) + "\n")


def evaluate(model, data, split_name: str = "test") -> dict:
    import torch
    ms_all = data["ms"]
    ms = ms_all[:, :HEURISTIC_COL]
    tr, te = split(data["meta"])
    sel = te if split_name == "test" else tr
    X = torch.from_numpy(data["features"][sel].astype(np.float32)).cuda()
    pred = model.forward(X).cpu().numpy()
    picks = learned_picks(pred, ms[sel])
    r_learn = regrets(picks, ms[sel])
    r_heur = regrets(None, ms[sel], ms_pick=ms_all[sel, HEURISTIC_COL])
    di = default_index()
    r_def = regrets(np.full(sel.sum(), di), ms[sel])
    r_fb, n_fb = fallback_regrets(pred, ms[sel])
    best = np.where(ms[sel] > 0, ms[sel], np.inf).argmin(1)

    def stats(r):
        return {"mean": float(np.mean(r)), "p95": float(np.percentile(r, 95)), "max": float(np.max(r))}

    return {"split": split_name, "matrices": int(sel.sum()), "learned_regret": stats(r_learn),
            "fallback_regret": stats(r_fb), "fallback_candidates_mean": float(n_fb.mean()),
            "fallback_timed_share": float((n_fb > 1).mean()),
            "heuristic_regret": stats(r_heur), "default_csr5_regret": stats(r_def),
            "top1_accuracy": float(np.mean(picks == best)),
            "autotune_seconds_median": float(np.median(data["meta"][sel, 6]))}


def evaluate_by_law(model, data) -> dict:
    """Held-out mean regret of the learned pick per generator law."""
    import torch
    ms = data["ms"][:, :HEURISTIC_COL]
    _, te = split(data["meta"])
    X = torch.from_numpy(data["features"][te].astype(np.float32)).cuda()
    picks = learned_picks(model.forward(X).cpu().numpy(), ms[te])
    r = regrets(picks, ms[te])
    laws = data["meta"][te, 1].astype(int)
    return {LAWS[k]: {"matrices": int((laws == k).sum()), "mean": float(r[laws == k].mean())}
            for k in sorted(set(laws.tolist()))}


def selection_cost(model, count: int = 8, max_rows: int = 2_000_000) -> dict:
    """Wall time of spmv_select(LEARNED) vs spmv_autotune on a few matrices."""
    import torch
    h = api.SpmvHandle()
    t_sel, t_fb, t_tune = [], [], []
    for seed in range(5, 5 + 5 * count, 5):
        spec, _, _ = spec_for_seed(seed, max_rows)
        A = selector.gen_device(spec)
        torch.cuda.synchronize()
        selector.select(h, A, selector.SELECT_LEARNED, model)  # warm
        t0 = time.perf_counter()
        for _ in range(10):
            selector.select(h, A, selector.SELECT_LEARNED, model)
        torch.cuda.synchronize()
        t_sel.append((time.perf_counter() - t0) / 10)
        t0 = time.perf_counter()
        selector.select(h, A, selector.SELECT_LEARNED_FALLBACK, model)
        torch.cuda.synchronize()
        t_fb.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        selector.autotune(h, A, None, repeats=0)
        torch.cuda.synchronize()
        t_tune.append(time.perf_counter() - t0)
        del A
    s, t = float(np.median(t_sel)), float(np.median(t_tune))
    return {"select_ms_median": s * 1e3, "autotune_ms_median": t * 1e3, "cost_ratio": t / s,
            "fallback_ms_mean": float(np.mean(t_fb)) * 1e3, "fallback_cost_ratio": t / float(np.mean(t_fb))}


def cmd_evaluate(a):
    data = load_corpus(a.corpus)
    model = selector.MLP.load(a.model)
    rep = {"test": evaluate(model, data, "test"), "train": evaluate(model, data, "train"),
           "by_law": evaluate_by_law(model, data)}
    if a.cost:
        rep["selection_cost"] = selection_cost(model)
    print(json.dumps(rep, indent=1))
    if a.report:
        Path(a.report).write_text(json.dumps(rep, indent=1) + "\n")


def main(argv=None):
    p = argparse.ArgumentParser(prog="python -m muxi_spmv_gb300.selector_train")
    sub = p.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("corpus")
    c.add_argument("--out", required=True)
    c.add_argument("--start", type=int, default=0)
    c.add_argument("--count", type=int, default=4000)
    c.add_argument("--chunk", type=int, default=100)
    c.add_argument("--max-rows", type=int, default=10_000_000)
    c.add_argument("--max-nnz", type=int, default=600_000_000)
    c.add_argument("--time-limit", type=float, default=0.0, help="seconds; stop after the chunk that passes it")
    r = sub.add_parser("relabel")
    r.add_argument("--corpus", required=True)
    r.add_argument("--index", type=int, required=True, help="variant space index to re-time")
    r.add_argument("--out", required=True, help="directory of resumable chunks")
    r.add_argument("--merged", required=True, help="corpus .npz written once every chunk is done")
    r.add_argument("--chunk", type=int, default=200)
    r.add_argument("--max-rows", type=int, default=10_000_000)
    r.add_argument("--max-nnz", type=int, default=600_000_000)
    r.add_argument("--time-limit", type=float, default=0.0, help="seconds; stop after the chunk that passes it")
    t = sub.add_parser("train")
    t.add_argument("--corpus", required=True)
    t.add_argument("--model", required=True)
    t.add_argument("--hidden", type=int, default=128)
    t.add_argument("--epochs", type=int, default=800)
    t.add_argument("--batch", type=int, default=128)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--report")
    t.add_argument("--merged", help="also write the combined records to this .npz")
    e = sub.add_parser("evaluate")
    e.add_argument("--corpus", required=True)
    e.add_argument("--model", required=True)
    e.add_argument("--cost", action="store_true")
    e.add_argument("--report")
    a = p.parse_args(argv)
    {"corpus": cmd_corpus, "relabel": cmd_relabel, "train": cmd_train, "evaluate": cmd_evaluate}[a.cmd](a)


if __name__ == "__main__":
    sys.exit(main())
