"""Shared fixtures.  `gpu`-marked tests need a CUDA device and the built
library; everything else runs on a CPU-only machine."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmuxispmv.so")
    config.addinivalue_line("markers", "refsrc: needs the reference source tree (oracle/_ref pinning)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def mx():
    import muxi_spmv_gb300 as m
    m.lib()  # builds if needed; raises if the library cannot be built
    return m


@pytest.fixture(scope="session")
def cuda(mx):
    if not has_gpu():
        pytest.fail("gpu test selected but no CUDA device is visible")
    import torch
    torch.cuda.init()
    return torch


@pytest.fixture(scope="session")
def handle(cuda, mx):
    h = mx.spmv_create_handle()
    yield h
    h.destroy()


def device_csr(mx, rp, ci, v, cols):
    A = mx.CSRMatrix(rp, ci, v, cols)
    A.copyToDevice()
    return A


def tol_for(dtype) -> float:
    # Per-row bound |y - y_ref| <= tol * sum_j |a_ij x_j| (FP32 1e-5, FP64 1e-13).
    return 1e-5 if dtype == np.float32 else 1e-13
