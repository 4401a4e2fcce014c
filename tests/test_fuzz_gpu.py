"""Seeded random matrices through every kernel family, against the FP64
oracle at the strict per-row bound (FP32 1e-5, FP64 1e-13 of sum |a x|).

Each seed draws a shape (square or not, 1 to 40,000 rows), a row-length law
(Poisson, Zipf with rows of thousands of nonzeros, runs of empty rows, all
rows empty) and a column law (uniform, banded around the diagonal, clustered
near it with a uniform share, as the power-law benchmark matrix has), then
runs the AUTO plan, each plan-only kernel shape, the CSR row kernels, merge
path, ELL where its padding gate admits the matrix, and the stateless call.
The edge-case matrices of test_spmv_gpu.py pin the known corners; this file
looks for the ones nobody listed."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import device_csr, tol_for

pytestmark = pytest.mark.gpu

SEEDS = list(range(16))


def random_csr(seed: int):
    rng = np.random.default_rng(9000 + seed)
    R = int(np.exp(rng.uniform(0, np.log(40000))))
    C = R if rng.random() < 0.6 else max(1, int(R * np.exp(rng.uniform(-2, 2))))
    law = ("poisson", "zipf", "empty_runs", "all_empty")[seed % 4 if seed % 8 != 7 else 1]
    if law == "poisson":
        lens = rng.poisson(rng.uniform(1, 40), R)
    elif law == "zipf":
        lens = np.minimum(rng.zipf(rng.uniform(1.4, 2.2), R), rng.integers(50, 20000))
    elif law == "empty_runs":
        lens = rng.poisson(rng.uniform(2, 20), R) * (rng.random(R) < 0.3)
        if R > 10:
            lens[: R // 10] = 0
    else:
        lens = np.zeros(R, np.int64)
    lens = np.minimum(lens, C).astype(np.int64)
    rp = np.r_[0, np.cumsum(lens)].astype(np.int32)
    cols = []
    mode = rng.integers(0, 3)
    for r, l in enumerate(lens):
        if l == 0:
            continue
        if mode == 0 or l * 2 > C:  # uniform, without replacement
            c = rng.choice(C, int(l), replace=False)
        else:
            centre = int(r * C / max(R, 1))
            width = int(rng.integers(8, 4096)) if mode == 1 else 4096
            near = rng.integers(centre - width, centre + width + 1, int(l)) % C
            c = near if mode == 1 else np.where(rng.random(int(l)) < 0.7, near, rng.integers(0, C, int(l)))
            c = np.unique(c)
            while c.size < l:  # top up duplicates with fresh columns
                c = np.unique(np.r_[c, rng.integers(0, C, int(l) - c.size)])
        cols.append(np.sort(c))
    ci = (np.concatenate(cols) if cols else np.zeros(0)).astype(np.int32)
    v = rng.standard_normal(ci.size)
    return rp, ci, v, C, law


def _variants(mx):
    R = mx.RANGE_PER_RESIDENT_BLOCK
    return [None,
            mx.make_variant(mx.KERNEL_SCALAR, 256), mx.make_variant(mx.KERNEL_VECTOR, 256, 8, 0, 4),
            mx.make_variant(mx.KERNEL_VECTOR, 128, 32, 0, 1), mx.make_variant(mx.KERNEL_MERGE, 256, 0, 8, 4),
            mx.make_variant(mx.KERNEL_CSR5, 256, 0, 8, 1), mx.make_variant(mx.KERNEL_CSR5, 128, 0, 16, 32),
            mx.make_variant(mx.KERNEL_CSR5, 1024, R, 16, 32), mx.make_variant(mx.KERNEL_CSR5, 1024, R, 8, 64),
            mx.make_variant(mx.KERNEL_CSR5, 512, 3, 16, 64), mx.make_variant(mx.KERNEL_BAND, 512, 0, 16),
            mx.make_variant(mx.KERNEL_BAND, 1024, 25, 8, 14), mx.make_variant(mx.KERNEL_BAND, 1024, 2, 8, 1),
            mx.make_variant(mx.KERNEL_STREAM, 512), mx.make_variant(mx.KERNEL_ELL)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("seed", SEEDS)
def test_random_matrices_every_kernel(mx, cuda, handle, seed, dtype):
    torch = cuda
    rp, ci, v, C, law = random_csr(seed)
    v = v.astype(dtype)
    A = device_csr(mx, rp, ci, v, C)
    xh = np.random.default_rng(seed).uniform(-1, 1, C).astype(dtype)
    x = torch.from_numpy(xh).cuda()
    y_ref, absum = oracle.spmv_ref(rp, ci, v, xh)
    tol = tol_for(dtype)
    ran = 0
    for var in _variants(mx):
        if var is not None and dtype == np.float64 and var.kernel == mx.KERNEL_STREAM:
            continue  # FP64 stream shapes are listed in test_spmv_gpu.py
        try:
            p = mx.Plan(handle, A, var)
        except mx.SpmvError:
            assert var is not None and var.kernel == mx.KERNEL_ELL  # only ELL may refuse (padding gate)
            continue
        y = torch.full((A.numRows,), float("nan"), dtype=x.dtype, device="cuda")
        p.exec(x, y)
        torch.cuda.synchronize()
        assert p.device_error() == 0
        err = np.abs(y.cpu().numpy().astype(np.float64) - y_ref)
        bad = np.flatnonzero(~(err <= tol * absum))
        name = "auto" if var is None else str(var.as_dict())
        assert bad.size == 0, f"seed {seed} ({law}, {A.numRows}x{C}, nnz {A.nnz}) {name}: rows {bad[:5]}"
        p.destroy()
        ran += 1
    y = torch.full((A.numRows,), float("nan"), dtype=x.dtype, device="cuda")
    mx.spmv_csr(A, x, y)
    torch.cuda.synchronize()
    err = np.abs(y.cpu().numpy().astype(np.float64) - y_ref)
    assert (err <= tol * absum).all(), f"seed {seed} stateless"
    assert ran >= 10
