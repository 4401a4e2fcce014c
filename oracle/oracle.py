"""numpy front end of the C oracle (oracle.c).  Test infrastructure only."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_oracle import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int


def _declare(L):
    sig = {
        "oracle_spmv_f32": (None, [I, P, P, P, P, P, P, I]),
        "oracle_spmv_f64": (None, [I, P, P, P, P, P, P, I]),
        "oracle_cpu_spmv_f32": (None, [I, P, P, P, P, P, I]),
        "oracle_cpu_spmv_f64": (None, [I, P, P, P, P, P, I]),
        "oracle_csr5_tiles": (None, [I, I, P, I, P, P]),
        "oracle_merge_partitions": (None, [I, I, I, P]),
        "oracle_merge_search": (None, [P, I, I, P, I, P, P]),
        "oracle_merge_default_partitions": (I, [I, I]),
        "oracle_csr_to_ell_f32": (C.c_longlong, [I, P, P, P, I, P, P, P]),
        "oracle_csr_to_ell_f64": (C.c_longlong, [I, P, P, P, I, P, P, P]),
        "oracle_max_row_length": (I, [I, P]),
        "oracle_row_reorder_f32": (None, [I, P, P, P, P, P, P, P]),
        "oracle_restore_order_f32": (None, [I, P, P, P]),
        "oracle_colperm_center_of_mass": (None, [I, I, P, P, P, P]),
        "oracle_colperm_min_row": (None, [I, I, P, P, P, P]),
        "oracle_colperm_frequency": (None, [I, I, P, P, P]),
        "oracle_apply_colperm": (None, [I, I, P, P, P]),
        "oracle_permute_x_f32": (None, [I, P, P, P]),
        "oracle_sort_within_rows_f32": (None, [I, P, P, P]),
        "oracle_distinct_columns": (C.c_longlong, [I, C.c_longlong, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be contiguous"
    return a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def spmv_ref(rowPtr, colIdx, values, x, threads: int = 0):
    """FP64 compensated y and the per-row scale sum |a_ij x_j|."""
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    rows = len(rowPtr) - 1
    y = np.empty(rows, np.float64)
    a = np.empty(rows, np.float64)
    if values.dtype == np.float32:
        v, xx = np.ascontiguousarray(values), np.ascontiguousarray(x, np.float32)
        lib().oracle_spmv_f32(rows, _p(rowPtr), _p(colIdx), _p(v), _p(xx), _p(y), _p(a), threads)
    else:
        v, xx = np.ascontiguousarray(values, np.float64), np.ascontiguousarray(x, np.float64)
        lib().oracle_spmv_f64(rows, _p(rowPtr), _p(colIdx), _p(v), _p(xx), _p(y), _p(a), threads)
    return y, a


def cpu_spmv(rowPtr, colIdx, values, x, threads: int = 1, out=None):
    """The reference's CPU CSR loop (serial when threads == 1)."""
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    rows = len(rowPtr) - 1
    if values.dtype == np.float32:
        y = out if out is not None else np.empty(rows, np.float32)
        lib().oracle_cpu_spmv_f32(rows, _p(rowPtr), _p(colIdx), _p(values), _p(np.ascontiguousarray(x, np.float32)),
                                  _p(y), threads)
    else:
        y = out if out is not None else np.empty(rows, np.float64)
        lib().oracle_cpu_spmv_f64(rows, _p(rowPtr), _p(colIdx), _p(values), _p(np.ascontiguousarray(x, np.float64)),
                                  _p(y), threads)
    return y


def row_errors(y, y_ref, absum, tol: float):
    """Per-row |y - y_ref| / (tol * absum); a value <= 1 passes.  Rows whose
    scale is zero must match exactly (their bound is zero)."""
    err = np.abs(np.asarray(y, np.float64) - y_ref)
    bound = tol * absum
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(bound > 0, err / np.where(bound > 0, bound, 1.0), np.where(err > 0, np.inf, 0.0))
    return ratio


def csr5_tiles(rowPtr, nnz: int, sigma: int):
    rowPtr = _i32(rowPtr)
    rows = len(rowPtr) - 1
    T = (nnz + sigma - 1) // sigma
    trp = np.empty(T, np.int32)
    tno = np.empty(T, np.int32)
    lib().oracle_csr5_tiles(rows, nnz, _p(rowPtr), sigma, _p(trp), _p(tno))
    return trp, tno


def merge_partitions(rows: int, nnz: int, P: int):
    pos = np.empty(P + 1, np.int32)
    lib().oracle_merge_partitions(rows, nnz, P, _p(pos))
    return pos


def merge_search(rowPtr, nnz: int, diag):
    rowPtr, diag = _i32(rowPtr), _i32(diag)
    rows = len(rowPtr) - 1
    r = np.empty(len(diag), np.int32)
    z = np.empty(len(diag), np.int32)
    lib().oracle_merge_search(_p(rowPtr), rows, nnz, _p(diag), len(diag), _p(r), _p(z))
    return r, z


def merge_default_partitions(rows: int, nnz: int) -> int:
    return lib().oracle_merge_default_partitions(rows, nnz)


def csr_to_ell(rowPtr, colIdx, values, width: int = 0):
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    rows = len(rowPtr) - 1
    W = width if width > 0 else lib().oracle_max_row_length(rows, _p(rowPtr))
    ec = np.empty(rows * W, np.int32)
    ev = np.empty(rows * W, values.dtype)
    wout = C.c_int(0)
    f = lib().oracle_csr_to_ell_f32 if values.dtype == np.float32 else lib().oracle_csr_to_ell_f64
    trunc = f(rows, _p(rowPtr), _p(colIdx), _p(np.ascontiguousarray(values)), W, C.byref(wout), _p(ec), _p(ev))
    return ec, ev, wout.value, trunc


def row_reorder(rowPtr, colIdx, values):
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    values = np.ascontiguousarray(values, np.float32)
    rows = len(rowPtr) - 1
    rm = np.empty(rows, np.int32)
    nrp = np.empty(rows + 1, np.int32)
    nc = np.empty(len(colIdx), np.int32)
    nv = np.empty(len(colIdx), np.float32)
    lib().oracle_row_reorder_f32(rows, _p(rowPtr), _p(colIdx), _p(values), _p(rm), _p(nrp), _p(nc), _p(nv))
    return rm, nrp, nc, nv


def restore_order(y_perm, rowMap):
    y_perm = np.ascontiguousarray(y_perm, np.float32)
    rowMap = _i32(rowMap)
    y = np.empty_like(y_perm)
    lib().oracle_restore_order_f32(len(y), _p(y_perm), _p(rowMap), _p(y))
    return y


def colperm_center_of_mass(rowPtr, colIdx, cols: int):
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    fm = np.empty(cols, np.int32)
    key = np.empty(cols, np.float32)
    lib().oracle_colperm_center_of_mass(len(rowPtr) - 1, cols, _p(rowPtr), _p(colIdx), _p(fm), _p(key))
    return fm, key


def colperm_min_row(rowPtr, colIdx, cols: int):
    rowPtr, colIdx = _i32(rowPtr), _i32(colIdx)
    perm = np.empty(cols, np.int32)
    key = np.empty(cols, np.int32)
    lib().oracle_colperm_min_row(len(rowPtr) - 1, cols, _p(rowPtr), _p(colIdx), _p(perm), _p(key))
    return perm, key


def colperm_frequency(colIdx, cols: int):
    colIdx = _i32(colIdx)
    perm = np.empty(cols, np.int32)
    key = np.empty(cols, np.int32)
    lib().oracle_colperm_frequency(cols, len(colIdx), _p(colIdx), _p(perm), _p(key))
    return perm, key


def apply_colperm(perm, colIdx):
    perm, colIdx = _i32(perm), _i32(colIdx)
    out = np.empty_like(colIdx)
    lib().oracle_apply_colperm(len(perm), len(colIdx), _p(perm), _p(colIdx), _p(out))
    return out


def permute_x(forwardMap, x):
    forwardMap = _i32(forwardMap)
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().oracle_permute_x_f32(len(forwardMap), _p(forwardMap), _p(x), _p(out))
    return out


def sort_within_rows(rowPtr, colIdx, values):
    rowPtr = _i32(rowPtr)
    c = _i32(colIdx).copy()
    v = np.ascontiguousarray(values, np.float32).copy()
    lib().oracle_sort_within_rows_f32(len(rowPtr) - 1, _p(rowPtr), _p(c), _p(v))
    return c, v


def distinct_columns(colIdx, cols: int) -> int:
    colIdx = _i32(colIdx)
    return lib().oracle_distinct_columns(cols, len(colIdx), _p(colIdx))
