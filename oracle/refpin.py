"""ctypes front end of oracle/_ref/libmuxi_ref.so: the reference's own
hot-path functions built from its sources by oracle/ref/build_ref.py.  Used
only to pin the oracle and to make golden fixtures; needs the reference tree
(not present on GPU machines)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .ref import build_ref

_lib = None
P = C.c_void_p
I = C.c_int


def available() -> bool:
    return build_ref.available()


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build_ref.build()))
        sig = {
            "ref_csr5_tiles": [P, I, I, I, P, P, I],
            "ref_merge_partitions": [I, I, I, P],
            "ref_merge_search": [P, I, I, P, I, P, P],
            "ref_cpu_spmv_f32": [I, P, P, P, P, P],
            "ref_cpu_spmv_f64": [I, P, P, P, P, P],
            "ref_rcm_perm": [I, I, I, P, P, P, P],
            "ref_frequency_perm": [I, I, I, P, P, P, P],
            "ref_row_reorder": [I, I, I, P, P, P, P, P, P, P],
            "ref_center_of_mass_perm": [I, I, I, P, P, P, P],
            "ref_sort_within_rows": [I, I, I, P, P, P],
            "ref_csr_to_ell": [I, I, I, P, P, P, I, P, P],
            "ref_mtx_read_f64": [C.c_char_p, I, P, P, P, P],
        }
        for n, a in sig.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = I if n in ("ref_csr_to_ell", "ref_mtx_read_f64") else None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _i(a):
    return np.ascontiguousarray(a, np.int32)


def csr5_tiles(rowPtr, nnz, sigma):
    rowPtr = _i(rowPtr)
    T = (nnz + sigma - 1) // sigma
    a, b = np.empty(T, np.int32), np.empty(T, np.int32)
    lib().ref_csr5_tiles(_p(rowPtr), len(rowPtr) - 1, nnz, sigma, _p(a), _p(b), T)
    return a, b


def merge_partitions(rows, nnz, P_):
    # The reference kernel's grid covers P+2 threads but writes only t <= P.
    pos = np.full(P_ + 1, -7, np.int32)
    lib().ref_merge_partitions(rows, nnz, P_, _p(pos))
    return pos


def merge_search(rowPtr, nnz, diag):
    rowPtr, diag = _i(rowPtr), _i(diag)
    r, z = np.empty(len(diag), np.int32), np.empty(len(diag), np.int32)
    lib().ref_merge_search(_p(rowPtr), len(rowPtr) - 1, nnz, _p(diag), len(diag), _p(r), _p(z))
    return r, z


def cpu_spmv(rowPtr, colIdx, values, x):
    rowPtr, colIdx = _i(rowPtr), _i(colIdx)
    rows = len(rowPtr) - 1
    if values.dtype == np.float32:
        y = np.empty(rows, np.float32)
        lib().ref_cpu_spmv_f32(rows, _p(rowPtr), _p(colIdx), _p(values), _p(np.ascontiguousarray(x, np.float32)), _p(y))
    else:
        y = np.empty(rows, np.float64)
        lib().ref_cpu_spmv_f64(rows, _p(rowPtr), _p(colIdx), _p(values), _p(np.ascontiguousarray(x, np.float64)), _p(y))
    return y


def _perm(fn, rowPtr, colIdx, cols):
    rowPtr, colIdx = _i(rowPtr), _i(colIdx)
    perm = np.empty(cols, np.int32)
    newc = np.empty(max(len(colIdx), 1), np.int32)
    fn(len(rowPtr) - 1, cols, len(colIdx), _p(rowPtr), _p(colIdx), _p(perm), _p(newc))
    return perm, newc[: len(colIdx)]


def rcm_perm(rowPtr, colIdx, cols):
    return _perm(lib().ref_rcm_perm, rowPtr, colIdx, cols)


def frequency_perm(rowPtr, colIdx, cols):
    return _perm(lib().ref_frequency_perm, rowPtr, colIdx, cols)


def center_of_mass_perm(rowPtr, colIdx, cols):
    return _perm(lib().ref_center_of_mass_perm, rowPtr, colIdx, cols)


def row_reorder(rowPtr, colIdx, values, cols):
    rowPtr, colIdx = _i(rowPtr), _i(colIdx)
    values = np.ascontiguousarray(values, np.float32)
    rows, n = len(rowPtr) - 1, len(colIdx)
    rm, nrp = np.empty(rows, np.int32), np.empty(rows + 1, np.int32)
    nc, nv = np.empty(max(n, 1), np.int32), np.empty(max(n, 1), np.float32)
    lib().ref_row_reorder(rows, cols, n, _p(rowPtr), _p(colIdx), _p(values), _p(rm), _p(nrp), _p(nc), _p(nv))
    return rm, nrp, nc[:n], nv[:n]


def sort_within_rows(rowPtr, colIdx, values, cols):
    rowPtr = _i(rowPtr)
    c = _i(colIdx).copy()
    v = np.ascontiguousarray(values, np.float32).copy()
    lib().ref_sort_within_rows(len(rowPtr) - 1, cols, len(c), _p(rowPtr), _p(c), _p(v))
    return c, v


def csr_to_ell(rowPtr, colIdx, values, cols, maxElements=0):
    rowPtr, colIdx = _i(rowPtr), _i(colIdx)
    values = np.ascontiguousarray(values, np.float32)
    rows = len(rowPtr) - 1
    W = maxElements if maxElements > 0 else int(np.max(np.diff(rowPtr))) if rows else 0
    ec = np.empty(max(rows * W, 1), np.int32)
    ev = np.empty(max(rows * W, 1), np.float32)
    w = lib().ref_csr_to_ell(rows, cols, len(colIdx), _p(rowPtr), _p(colIdx), _p(values), maxElements, _p(ec), _p(ev))
    return ec[: rows * w], ev[: rows * w], w


def mtx_read(path, expand=True):
    """The reference's readMTXFile<double> (src/generators/mtx_io.cu:111-222):
    (status, rowPtr, colIdx, values, numCols)."""
    dims = np.zeros(3, np.int32)
    st = lib().ref_mtx_read_f64(str(path).encode(), 1 if expand else 0, _p(dims), None, None, None)
    if st != 0:
        return st, None, None, None, 0
    rows, cols, nnz = (int(d) for d in dims)
    rp = np.empty(rows + 1, np.int32)
    ci = np.empty(max(nnz, 1), np.int32)
    v = np.empty(max(nnz, 1), np.float64)
    lib().ref_mtx_read_f64(str(path).encode(), 1 if expand else 0, _p(dims), _p(rp), _p(ci), _p(v))
    return 0, rp, ci[:nnz], v[:nnz], cols
