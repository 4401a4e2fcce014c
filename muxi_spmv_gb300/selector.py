"""Kernel selection over the C ABI: device-generated matrices, matrix
features, the exhaustive autotuner, the selector MLP and spmv_select.

The reference chooses a kernel with one fixed rule on the integer mean row
length (src/spmv/csr/spmv_csr.cu:115-153); that rule is SELECT_HEURISTIC here.
Everything else in this module is new: the autotuner labels a corpus, the MLP
(forward, backward and Adam are CUDA kernels in the library) learns to predict
each variant's slowdown from 32 features, and spmv_select / set_selector put
the prediction behind the plan API.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import (NUM_FEATURES, SELECT_AUTOTUNE, SELECT_HEURISTIC, SELECT_LEARNED,  # noqa: F401
                   SELECT_LEARNED_TOPK, SELECT_LEARNED_FALLBACK, FALLBACK_MARGIN, FALLBACK_MAX, SPMV_TYPE_DOUBLE, SPMV_TYPE_FLOAT, GenParams, Variant, check, lib)
from .api import GenSpec, SpmvHandle, _ptr, _stream_ptr, _torch

DEFAULT_MODEL = Path(__file__).resolve().parent / "data" / "selector_gb300.mxsmlp"


@dataclass
class DeviceCSR:
    """A CSR matrix that exists only in device memory (torch tensors).
    Accepted wherever the api module takes a CSRMatrix on the device side
    (Plan, spmv_csr, ...)."""
    numRows: int
    numCols: int
    nnz: int
    d_rowPtr: object
    d_colIdx: object
    d_values: object

    @property
    def dtype(self):
        torch = _torch()
        return np.float32 if self.d_values.dtype == torch.float32 else np.float64

    def device_args(self):
        return (self.numRows, self.numCols, self.nnz, _ptr(self.d_rowPtr), _ptr(self.d_colIdx),
                _ptr(self.d_values))

    @property
    def type_code(self) -> int:
        return SPMV_TYPE_FLOAT if self.dtype == np.float32 else SPMV_TYPE_DOUBLE

    def nbytes(self) -> int:
        vs = 4 if self.dtype == np.float32 else 8
        return self.nnz * (vs + 4) + (self.numRows + 1) * 4


def gen_device(spec: GenSpec, stream=None) -> DeviceCSR:
    """Generates `spec` on the device (laws POISSON_UNIFORM, ZIPF_UNIFORM,
    BANDED, BLOCKDIAG, STENCIL2D, STENCIL3D); FP32."""
    torch = _torch()
    p = spec.params()
    s = _stream_ptr(stream)
    rowPtr = torch.empty(spec.numRows + 1, dtype=torch.int32, device="cuda")
    nnz = C.c_longlong()
    check(lib().spmv_gen_device_row_ptr(C.byref(p), _ptr(rowPtr), C.byref(nnz), s), "spmv_gen_device_row_ptr")
    n = nnz.value
    colIdx = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    values = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
    check(lib().spmv_gen_device_fill_f32(C.byref(p), _ptr(rowPtr), _ptr(colIdx), _ptr(values), s),
          "spmv_gen_device_fill_f32")
    return DeviceCSR(spec.numRows, spec.numCols, n, rowPtr, colIdx, values)


def gen_device_vector(n: int, seed: int, lo: float = -1.0, hi: float = 1.0, stream=None):
    torch = _torch()
    out = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
    check(lib().spmv_gen_device_vector_f32(n, seed, lo, hi, _ptr(out), _stream_ptr(stream)),
          "spmv_gen_device_vector_f32")
    return out[:n]


def matrix_features(A, stream=None):
    """The 32 selector features of a device CSR matrix, as a device tensor."""
    torch = _torch()
    f = torch.empty(NUM_FEATURES, dtype=torch.float32, device="cuda")
    t = SPMV_TYPE_FLOAT if A.dtype == np.float32 else SPMV_TYPE_DOUBLE
    check(lib().spmv_matrix_features(t, A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(f),
                                     _stream_ptr(stream)), "spmv_matrix_features")
    return f


def variant_space() -> list[Variant]:
    n = lib().spmv_variant_space(None, 0)
    arr = (Variant * n)()
    lib().spmv_variant_space(arr, n)
    return [arr[i] for i in range(n)]


def variant_name(v: Variant) -> str:
    k = {1: "scalar", 2: "vector", 3: "merge", 4: "csr5", 5: "ell", 6: "heuristic", 7: "band", 8: "stream",
         0: "auto"}
    name = k.get(v.kernel, str(v.kernel))
    if v.kernel == 2:
        return f"vector_b{v.blockSize}_t{v.threadsPerRow}"
    if v.kernel == 4 and v.threadsPerRow > 0:  # CSR5 block ranges (prefetching with vectorWidth 64)
        per = "sm" if v.threadsPerRow >= _lib.RANGE_PER_RESIDENT_BLOCK else str(v.threadsPerRow)
        pf = "_pf" if v.vectorWidth == _lib.CSR5_ORDERED_PREFETCH else ""
        return f"csr5r_b{v.blockSize}_e{v.itemsPerThread}_r{per}{pf}"
    if v.kernel == 8:
        return f"stream_b{v.blockSize}_e{v.itemsPerThread}_s{v.threadsPerRow}"
    if v.kernel == 7:  # window kernel: tiles per warp of a range, window in 1,024-element units
        return f"band_b{v.blockSize}_e{v.itemsPerThread}_t{v.threadsPerRow}_w{v.vectorWidth}"
    if v.kernel in (3, 4, 7):
        return f"{name}_b{v.blockSize}_e{v.itemsPerThread}"
    return f"{name}_b{v.blockSize}"


def autotune(handle: SpmvHandle, A, candidates: list[Variant] | None = None, repeats: int = 0):
    """Times each candidate (default: the whole space) as a plan on A.
    repeats <= 0 sizes each variant's timing loop to about 2 ms.
    Returns (ms per candidate as numpy, -1 where it does not apply; best index)."""
    t = SPMV_TYPE_FLOAT if A.dtype == np.float32 else SPMV_TYPE_DOUBLE
    if candidates is None:
        arr, n = None, lib().spmv_variant_space(None, 0)
    else:
        n = len(candidates)
        arr = (Variant * n)(*candidates)
    ms = np.empty(n, np.float32)
    best = C.c_int(-1)
    check(lib().spmv_autotune(handle.raw, t, *A.device_args(), arr, n, repeats, ms.ctypes.data_as(C.c_void_p),
                              C.byref(best)), "spmv_autotune")
    return ms, best.value


class MLP:
    """The selector network (CUDA forward/backward/Adam in the library)."""

    def __init__(self, inp: int = NUM_FEATURES, h1: int = 128, h2: int = 128, out: int | None = None,
                 seed: int = 0, _raw=None):
        if _raw is not None:
            self._m = _raw
        else:
            if out is None:
                out = lib().spmv_variant_space(None, 0)
            m = C.c_void_p()
            check(lib().spmv_mlp_create(inp, h1, h2, out, seed, C.byref(m)), "spmv_mlp_create")
            self._m = m

    @property
    def raw(self):
        return self._m

    @classmethod
    def load(cls, path) -> "MLP":
        m = C.c_void_p()
        check(lib().spmv_mlp_load(str(path).encode(), C.byref(m)), "spmv_mlp_load")
        return cls(_raw=m)

    def save(self, path):
        check(lib().spmv_mlp_save(self._m, str(path).encode()), "spmv_mlp_save")

    @property
    def num_params(self) -> int:
        return lib().spmv_mlp_num_params(self._m)

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        check(lib().spmv_mlp_get_params(self._m, p.ctypes.data_as(C.c_void_p), p.size), "spmv_mlp_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().spmv_mlp_set_params(self._m, p.ctypes.data_as(C.c_void_p), p.size), "spmv_mlp_set_params")

    def set_normalization(self, mean: np.ndarray, std: np.ndarray):
        mean = np.ascontiguousarray(mean, np.float32)
        std = np.ascontiguousarray(std, np.float32)
        check(lib().spmv_mlp_set_normalization(self._m, mean.ctypes.data_as(C.c_void_p),
                                               std.ctypes.data_as(C.c_void_p)), "spmv_mlp_set_normalization")

    @property
    def shape(self) -> tuple[int, int, int, int]:
        """(in, h1, h2, out)."""
        d = [C.c_int() for _ in range(4)]
        check(lib().spmv_mlp_shape(self._m, *[C.byref(x) for x in d]), "spmv_mlp_shape")
        return tuple(x.value for x in d)

    def forward(self, X, stream=None):
        """X: device float32 tensor [batch, in] -> device tensor [batch, out]."""
        torch = _torch()
        X = X.contiguous()
        Y = torch.empty(X.shape[0], self.shape[3], dtype=torch.float32, device="cuda")
        check(lib().spmv_mlp_forward(self._m, _ptr(X), _ptr(Y), X.shape[0], _stream_ptr(stream)),
              "spmv_mlp_forward")
        return Y

    def gradients(self, X, T, M, stream=None):
        """(loss, host gradient vector) for one batch; no update."""
        g = np.empty(self.num_params, np.float32)
        loss = C.c_float()
        check(lib().spmv_mlp_gradients(self._m, _ptr(X), _ptr(T), _ptr(M), X.shape[0], C.byref(loss),
                                       g.ctypes.data_as(C.c_void_p), _stream_ptr(stream)), "spmv_mlp_gradients")
        return loss.value, g

    def train_step(self, X, T, M, lr: float, stream=None, want_loss: bool = False):
        loss = C.c_float()
        check(lib().spmv_mlp_train_step(self._m, _ptr(X), _ptr(T), _ptr(M), X.shape[0], lr,
                                        C.byref(loss) if want_loss else None, _stream_ptr(stream)),
              "spmv_mlp_train_step")
        return loss.value if want_loss else None

    def destroy(self):
        if self._m:
            check(lib().spmv_mlp_destroy(self._m), "spmv_mlp_destroy")
            self._m = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def select(handle: SpmvHandle, A, mode: int = SELECT_LEARNED, model: MLP | None = None, topK: int = 0):
    """spmv_select: (chosen Variant, index into variant_space() or -1)."""
    v = Variant()
    idx = C.c_int(-1)
    t = SPMV_TYPE_FLOAT if A.dtype == np.float32 else SPMV_TYPE_DOUBLE
    check(lib().spmv_select(handle.raw, mode, model.raw if model is not None else None, topK, t, *A.device_args(),
                            C.byref(v), C.byref(idx)), "spmv_select")
    return v, idx.value


def set_selector(handle: SpmvHandle, model: MLP | None, mode: int = SELECT_LEARNED):
    """Makes AUTO plans on `handle` use `model` (None clears it); mode
    SELECT_LEARNED_FALLBACK also times the variants predicted within 12%
    (at most 4 candidates)."""
    check(lib().spmv_set_selector(handle.raw, model.raw if model is not None else None), "spmv_set_selector")
    check(lib().spmv_set_selector_mode(handle.raw, mode), "spmv_set_selector_mode")


__all__ = ["DeviceCSR", "gen_device", "gen_device_vector", "matrix_features", "variant_space", "variant_name",
           "autotune", "MLP", "select", "set_selector", "DEFAULT_MODEL", "SELECT_HEURISTIC", "SELECT_LEARNED",
           "SELECT_AUTOTUNE", "SELECT_LEARNED_TOPK", "SELECT_LEARNED_FALLBACK", "FALLBACK_MARGIN", "FALLBACK_MAX", "NUM_FEATURES"]
