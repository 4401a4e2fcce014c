"""Batched SpMV / SpMM over many independent CSR matrices (spmv_batch_* in
the C ABI), and the uneven-batch workload: 1,024 square matrices with rows
log-uniform in [1,024, 262,144], mean row length uniform in [2, 64] with
Poisson or Zipf(2.0) row lengths, columns uniform, values N(0,1), X entries
U[-1,1], k right-hand sides in {1, 2, 4, 8, 16}.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from ._lib import (BATCH_LOOP, BATCH_LOOP_GRAPH, BATCH_PERSISTENT, BATCH_PERSISTENT_GRAPH,  # noqa: F401
                   BatchMatrix, BatchVariant, check, lib)
from .api import GEN_POISSON_UNIFORM, GEN_ZIPF_UNIFORM, GenSpec, SpmvHandle, _ptr, _torch


class BatchPlan:
    """A batch of device CSR matrices (CSRMatrix on the device or DeviceCSR)
    bound to k right-hand sides."""

    def __init__(self, handle: SpmvHandle, mats, k: int, variant: dict | None = None):
        self.handle = handle
        self.mats = list(mats)  # keeps the borrowed arrays alive
        self.k = k
        arr = (BatchMatrix * len(self.mats))()
        for i, A in enumerate(self.mats):
            arr[i] = BatchMatrix(A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(A.d_values))
        b = C.c_void_p()
        v = BatchVariant(**(variant or {}))
        check(lib().spmv_batch_create_ex(handle.raw, len(self.mats), arr, k, C.byref(v), C.byref(b)),
              "spmv_batch_create_ex")
        self._b = b
        self.xs = self.ys = None

    def set_vectors(self, xs, ys):
        """xs[i]: device float32 tensor numCols_i * k; ys[i]: numRows_i * k (row-major)."""
        n = len(self.mats)
        xa = (C.c_void_p * n)(*[_ptr(x) for x in xs])
        ya = (C.c_void_p * n)(*[_ptr(y) for y in ys])
        check(lib().spmv_batch_set_vectors_f32(self._b, xa, ya), "spmv_batch_set_vectors_f32")
        self.xs, self.ys = list(xs), list(ys)

    def exec(self, alpha: float = 1.0, beta: float = 0.0, mode: int = BATCH_PERSISTENT_GRAPH):
        check(lib().spmv_batch_exec_f32(self.handle.raw, self._b, alpha, beta, mode), "spmv_batch_exec_f32")

    @property
    def variant(self) -> dict:
        v = BatchVariant()
        check(lib().spmv_batch_get_variant(self._b, C.byref(v)), "spmv_batch_get_variant")
        return v.as_dict()

    def info(self):
        t, w, n = C.c_longlong(), C.c_int(), C.c_longlong()
        check(lib().spmv_batch_info(self._b, C.byref(t), C.byref(w), C.byref(n)), "spmv_batch_info")
        return {"tiles": t.value, "warps": w.value, "nnz": n.value}

    def destroy(self):
        if self._b:
            check(lib().spmv_batch_destroy(self._b), "spmv_batch_destroy")
            self._b = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class BatchGroupPlan:
    """Matrices with their own number of right-hand sides ks[i] (1, 2, 4, 8
    or 16): one batch per distinct k, run back to back (one graph in the
    graph modes).  variants: None or {k: variant dict}."""

    def __init__(self, handle: SpmvHandle, mats, ks, variants: dict | None = None):
        self.handle = handle
        self.mats = list(mats)
        self.ks = [int(k) for k in ks]
        n = len(self.mats)
        arr = (BatchMatrix * n)()
        for i, A in enumerate(self.mats):
            arr[i] = BatchMatrix(A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(A.d_values))
        karr = (C.c_int * n)(*self.ks)
        vp = None
        if variants:
            va = (BatchVariant * 5)(*[BatchVariant(**variants.get(k, {})) for k in (1, 2, 4, 8, 16)])
            vp = va
        g = C.c_void_p()
        check(lib().spmv_batch_group_create(handle.raw, n, arr, karr, vp, C.byref(g)), "spmv_batch_group_create")
        self._g = g

    def set_vectors(self, xs, ys):
        n = len(self.mats)
        xa = (C.c_void_p * n)(*[_ptr(x) for x in xs])
        ya = (C.c_void_p * n)(*[_ptr(y) for y in ys])
        check(lib().spmv_batch_group_set_vectors_f32(self._g, xa, ya), "spmv_batch_group_set_vectors_f32")
        self.xs, self.ys = list(xs), list(ys)

    def exec(self, alpha: float = 1.0, beta: float = 0.0, mode: int = BATCH_PERSISTENT_GRAPH):
        check(lib().spmv_batch_group_exec_f32(self.handle.raw, self._g, alpha, beta, mode),
              "spmv_batch_group_exec_f32")

    def info(self):
        b, n = C.c_int(), C.c_longlong()
        check(lib().spmv_batch_group_info(self._g, C.byref(b), C.byref(n)), "spmv_batch_group_info")
        return {"batches": b.value, "nnz": n.value}

    def destroy(self):
        if self._g:
            check(lib().spmv_batch_group_destroy(self._g), "spmv_batch_group_destroy")
            self._g = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def batch_variant_space(k: int) -> list[dict]:
    """Launch shapes the batch autotuner times for k right-hand sides."""
    out = []
    for e, b in ((8, 2), (4, 2), (4, 3)):
        for c in (1024, 2048, 4096):
            out.append({"nnzPerSlot": e, "blocksPerSM": b, "chunkNnz": c, "ordered": 0})
    if k == 1:  # one warp per CSR5 tile, gathers in nonzero order
        out += [{"nnzPerSlot": e, "blocksPerSM": b, "chunkNnz": 0, "ordered": 1}
                for e, b in ((16, 10), (16, 8), (8, 16), (8, 12))]
    return out


def autotune_batch(handle: SpmvHandle, mats, k: int, xs, ys, candidates=None, repeats: int = 5,
                   stream=None):
    """Times each candidate variant (persistent graph launch) on this batch;
    returns (best variant, {variant key: ms})."""
    torch = _torch()
    cands = candidates or batch_variant_space(k)
    times = {}
    for v in cands:
        plan = BatchPlan(handle, mats, k, v)
        plan.set_vectors(xs, ys)
        plan.exec(1.0, 0.0, BATCH_PERSISTENT_GRAPH)
        s = stream or torch.cuda.current_stream()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(repeats):
            plan.exec(1.0, 0.0, BATCH_PERSISTENT_GRAPH)
        e1.record(s)
        e1.synchronize()
        times[(v["nnzPerSlot"], v["blocksPerSM"], v["chunkNnz"], v.get("ordered", 0))] = e0.elapsed_time(e1) / repeats
        plan.destroy()
    best = min(times, key=times.get)
    return {"nnzPerSlot": best[0], "blocksPerSM": best[1], "chunkNnz": best[2], "ordered": best[3]}, times


def _zipf_mean(s: float, K: int) -> float:
    k = np.arange(1, K + 1, dtype=np.float64)
    w = k ** (-s)
    return float((w * k).sum() / w.sum())


@dataclass
class BatchMatrixSpec:
    spec: GenSpec
    law: str
    mean_target: float


def uneven_specs(count: int = 1024, seed: int = 0, rmin: int = 1024, rmax: int = 262144):
    """Seeded per-matrix generator specs of the uneven batch."""
    rng = np.random.default_rng(np.random.SeedSequence([0xBA7C4, seed]))
    out = []
    for i in range(count):
        R = int(round(math.exp(rng.uniform(math.log(rmin), math.log(rmax)))))
        m = float(rng.uniform(2.0, 64.0))
        gseed = (seed << 20) + i + 1
        if rng.random() < 0.5:
            s = GenSpec(GEN_POISSON_UNIFORM, R, R, m, 0.0, float(min(R, int(4 * m + 64))), 0.0, gseed)
            out.append(BatchMatrixSpec(s, "poisson", m))
        else:
            cap = min(R, 65536)
            full = _zipf_mean(2.0, cap)
            if m <= full:
                k = np.arange(1, cap + 1, dtype=np.float64)
                w = k ** -2.0
                means = np.cumsum(w * k) / np.cumsum(w)
                clip = max(1, min(cap, int(np.searchsorted(means, m, side="right"))))
                off = 0.0
            else:
                clip, off = cap, float(round(m - full))
            s = GenSpec(GEN_ZIPF_UNIFORM, R, R, 2.0, float(clip), off, 0.0, gseed)
            out.append(BatchMatrixSpec(s, "zipf", m))
    return out


def build_uneven_batch(count: int = 1024, k: int = 1, seed: int = 0, rmin: int = 1024, rmax: int = 262144):
    """Generates the batch on the device: (matrices, xs, ys, specs)."""
    from .selector import gen_device, gen_device_vector
    torch = _torch()
    specs = uneven_specs(count, seed, rmin, rmax)
    mats, xs, ys = [], [], []
    for i, bs in enumerate(specs):
        A = gen_device(bs.spec)
        mats.append(A)
        xs.append(gen_device_vector(A.numCols * k, (seed << 24) + 7919 * i + 3, -1.0, 1.0))
        ys.append(torch.zeros(max(A.numRows * k, 1), dtype=torch.float32, device="cuda"))
    return mats, xs, ys, specs


__all__ = ["BatchPlan", "BatchGroupPlan", "uneven_specs", "build_uneven_batch", "batch_variant_space", "autotune_batch", "BATCH_PERSISTENT", "BATCH_PERSISTENT_GRAPH",
           "BATCH_LOOP", "BATCH_LOOP_GRAPH"]
