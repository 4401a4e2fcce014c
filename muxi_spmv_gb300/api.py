"""Python mirror of the muxi_spmv interface over the C ABI.

Names, argument order and meaning follow the reference's C++ API
(src/api/spmv_api.h, src/spmv/csr/spmv_csr.cuh, src/spmv/csr5/spmv_csr5.cuh,
src/formats/sparse_formats.h) so tests read like the reference's own.  Device
memory is held in torch tensors (plumbing only); every computation runs in
libmuxispmv.so.  Errors raise SpmvError carrying the spmv_status_t.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import (GenParams, Opts, SpmvError, Variant, check, lib, KERNEL_AUTO, KERNEL_SCALAR,  # noqa: F401
                   KERNEL_BAND, KERNEL_STREAM, CSR5_ORDERED, CSR5_ORDERED_PREFETCH, RANGE_PER_RESIDENT_BLOCK,
                   KERNEL_VECTOR, KERNEL_MERGE, KERNEL_CSR5, KERNEL_ELL, KERNEL_HEURISTIC,
                   SPMV_TYPE_FLOAT, SPMV_TYPE_DOUBLE, SPMV_OP_NORMAL, SPMV_OP_TRANSPOSE,
                   SPMV_FORMAT_CSR, SPMV_FORMAT_COO, SPMV_FORMAT_CSR2, SPMV_FORMAT_BSR, SPMV_FORMAT_CSR5,
                   SPMV_FORMAT_ELL)


def _torch():
    import torch
    return torch


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    """Accepts None (current torch stream), a torch.cuda.Stream or a raw handle."""
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream or None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def spmv_default_opts(stream=None, sync: bool = False) -> Opts:
    o = lib().spmv_default_opts()
    o.stream = _stream_ptr(stream)
    o.sync = 1 if sync else 0
    return o


# ---------------------------------------------------------------------------
# Matrices
# ---------------------------------------------------------------------------
class CSRMatrix:
    """CSRMatrix<T> (src/formats/sparse_formats.h:24-103): host arrays
    (rowPtr, colIdx, values as numpy) and device arrays (d_* as torch
    tensors).  The device arrays are owned by torch."""

    def __init__(self, rowPtr, colIdx, values, numCols: int):
        self.rowPtr = np.ascontiguousarray(rowPtr, np.int32)
        self.colIdx = np.ascontiguousarray(colIdx, np.int32)
        self.values = np.ascontiguousarray(values)
        if self.values.dtype not in (np.float32, np.float64):
            raise TypeError("values must be float32 or float64")
        self.numRows = len(self.rowPtr) - 1
        self.numCols = int(numCols)
        self.nnz = int(self.rowPtr[-1]) if self.numRows >= 0 and len(self.rowPtr) else 0
        self.d_rowPtr = self.d_colIdx = self.d_values = None

    @property
    def dtype(self):
        return self.values.dtype

    def allocateDevice(self, device="cuda"):
        torch = _torch()
        tdt = torch.float32 if self.dtype == np.float32 else torch.float64
        self.d_rowPtr = torch.empty(self.numRows + 1, dtype=torch.int32, device=device)
        self.d_colIdx = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=device)
        self.d_values = torch.empty(max(self.nnz, 1), dtype=tdt, device=device)
        return self

    def copyToDevice(self, device="cuda"):
        torch = _torch()
        if self.d_rowPtr is None:
            self.allocateDevice(device)
        self.d_rowPtr.copy_(torch.from_numpy(self.rowPtr))
        if self.nnz:
            self.d_colIdx[: self.nnz].copy_(torch.from_numpy(self.colIdx))
            self.d_values[: self.nnz].copy_(torch.from_numpy(self.values))
        return self

    def device_args(self):
        return (self.numRows, self.numCols, self.nnz, _ptr(self.d_rowPtr), _ptr(self.d_colIdx),
                _ptr(self.d_values))


# ---------------------------------------------------------------------------
# Handle (src/api/spmv_api.h:18-43)
# ---------------------------------------------------------------------------
class SpmvHandle:
    def __init__(self):
        h = C.POINTER(_lib.Handle)()
        check(lib().spmv_create_handle(C.byref(h)), "spmv_create_handle")
        self._h = h

    @property
    def raw(self):
        return self._h

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        return getattr(self._h.contents, name)

    def set_stream(self, stream):
        check(lib().spmv_set_stream(self._h, _stream_ptr(stream)), "spmv_set_stream")

    def destroy(self):
        if self._h:
            check(lib().spmv_destroy_handle(self._h), "spmv_destroy_handle")
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def spmv_create_handle() -> SpmvHandle:
    return SpmvHandle()


def spmv_destroy_handle(h: SpmvHandle):
    h.destroy()


def spmv_set_stream(h: SpmvHandle, stream):
    h.set_stream(stream)


# ---------------------------------------------------------------------------
# Execution
# ---------------------------------------------------------------------------
def _is_f32(A: CSRMatrix) -> bool:
    return A.dtype == np.float32


def spmv_csr(A: CSRMatrix, x, y, alpha=1.0, beta=0.0, opts: Opts | None = None):
    """spmv_csr<T> (src/spmv/csr/spmv_csr.cu:52-249) with alpha/beta applied."""
    o = opts if opts is not None else spmv_default_opts()
    f = lib().spmv_csr_f32 if _is_f32(A) else lib().spmv_csr_f64
    check(f(*A.device_args(), _ptr(x), _ptr(y), alpha, beta, C.byref(o)), "spmv_csr")
    return y


class COOMatrix:
    """COOMatrix<T> (src/formats/sparse_formats.h:113-162): host arrays rowIdx,
    colIdx, values (numpy) and device copies d_* (torch)."""

    def __init__(self, rowIdx, colIdx, values, numRows: int, numCols: int):
        self.rowIdx = np.ascontiguousarray(rowIdx, np.int32)
        self.colIdx = np.ascontiguousarray(colIdx, np.int32)
        self.values = np.ascontiguousarray(values)
        self.numRows, self.numCols, self.nnz = int(numRows), int(numCols), len(self.values)
        self.d_rowIdx = self.d_colIdx = self.d_values = None

    def copyToDevice(self, device="cuda"):
        torch = _torch()
        self.d_rowIdx = torch.from_numpy(self.rowIdx.copy() if self.nnz else np.zeros(1, np.int32)).to(device)
        self.d_colIdx = torch.from_numpy(self.colIdx.copy() if self.nnz else np.zeros(1, np.int32)).to(device)
        self.d_values = torch.from_numpy(self.values.copy() if self.nnz else np.zeros(1, self.values.dtype)).to(device)
        return self

    def device_args(self):
        return (self.numRows, self.numCols, self.nnz, _ptr(self.d_rowIdx), _ptr(self.d_colIdx), _ptr(self.d_values))


def coo_to_csr(A: COOMatrix, stream=None) -> CSRMatrix:
    """Device CSR of a COO matrix (entries ordered by row, then column)."""
    torch = _torch()
    dev = A.d_values.device
    rp = torch.empty(A.numRows + 1, dtype=torch.int32, device=dev)
    ci = torch.empty(max(A.nnz, 1), dtype=torch.int32, device=dev)
    va = torch.empty(max(A.nnz, 1), dtype=A.d_values.dtype, device=dev)
    f = lib().spmv_coo_to_csr_f32 if A.values.dtype == np.float32 else lib().spmv_coo_to_csr_f64
    check(f(*A.device_args(), _ptr(rp), _ptr(ci), _ptr(va), _stream_ptr(stream)), "spmv_coo_to_csr")
    B = CSRMatrix(np.zeros(A.numRows + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, A.values.dtype), A.numCols)
    B.nnz = A.nnz
    B.d_rowPtr, B.d_colIdx, B.d_values = rp, ci, va
    return B


def spmv_coo(A: COOMatrix, x, y, alpha=1.0, beta=0.0, opts: Opts | None = None):
    """y = alpha*A*x + beta*y for a COO matrix (converted per call)."""
    o = opts if opts is not None else spmv_default_opts()
    f = lib().spmv_coo_f32 if A.values.dtype == np.float32 else lib().spmv_coo_f64
    check(f(*A.device_args(), _ptr(x), _ptr(y), alpha, beta, C.byref(o)), "spmv_coo")
    return y


class BSRMatrix:
    """BSRMatrix<T, B> (src/formats/sparse_formats.h:207-269) on the device:
    d_rowPtr (block rows + 1), d_colIdx (block columns), d_values (dense
    B x B blocks, row-major)."""

    def __init__(self, numRows: int, numCols: int, blockSize: int, numBlocks: int, d_rowPtr, d_colIdx, d_values):
        self.numRows, self.numCols, self.blockSize, self.numBlocks = numRows, numCols, blockSize, numBlocks
        self.numBlockRows = (numRows + blockSize - 1) // blockSize
        self.numBlockCols = (numCols + blockSize - 1) // blockSize
        self.d_rowPtr, self.d_colIdx, self.d_values = d_rowPtr, d_colIdx, d_values


def csr_to_bsr(A: CSRMatrix, blockSize: int, stream=None) -> BSRMatrix:
    """Device BSR of a CSR matrix whose columns are sorted within rows."""
    torch = _torch()
    dev = A.d_values.device
    B = int(blockSize)
    nbr = (A.numRows + B - 1) // B
    rp = torch.empty(nbr + 1, dtype=torch.int32, device=dev)
    nb = C.c_int()
    check(lib().spmv_csr_to_bsr_count(A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), B, _ptr(rp),
                                      C.byref(nb), _stream_ptr(stream)), "spmv_csr_to_bsr_count")
    ci = torch.empty(max(nb.value, 1), dtype=torch.int32, device=dev)
    va = torch.empty(max(nb.value * B * B, 1), dtype=A.d_values.dtype, device=dev)
    f = lib().spmv_csr_to_bsr_f32 if _is_f32(A) else lib().spmv_csr_to_bsr_f64
    check(f(*A.device_args(), B, _ptr(rp), _ptr(ci), _ptr(va), _stream_ptr(stream)), "spmv_csr_to_bsr")
    return BSRMatrix(A.numRows, A.numCols, B, nb.value, rp, ci, va)


def spmv_bsr(M: BSRMatrix, x, y, alpha=1.0, beta=0.0, stream=None):
    """y = alpha*A*x + beta*y for a BSR matrix."""
    torch = _torch()
    f = lib().spmv_bsr_f32 if M.d_values.dtype == torch.float32 else lib().spmv_bsr_f64
    check(f(M.numRows, M.numCols, M.blockSize, M.numBlockRows, _ptr(M.d_rowPtr), _ptr(M.d_colIdx), _ptr(M.d_values),
            _ptr(x), _ptr(y), alpha, beta, _stream_ptr(stream)), "spmv_bsr")
    return y


def spmv_csr_transpose(A: CSRMatrix, x, y, alpha=1.0, beta=0.0, stream=None):
    """y = alpha*A^T*x + beta*y (the reference's spmv_exec_transpose, spmv_api.h:70-78)."""
    o = spmv_default_opts(stream)
    o.operation = _lib.SPMV_OP_TRANSPOSE
    f = lib().spmv_csr_f32 if _is_f32(A) else lib().spmv_csr_f64
    check(f(*A.device_args(), _ptr(x), _ptr(y), alpha, beta, C.byref(o)), "spmv_csr (transpose)")
    return y


def csr_transpose(A: CSRMatrix, stream=None) -> CSRMatrix:
    """CSR of A^T built on the device (host arrays left empty)."""
    torch = _torch()
    tdt = torch.float32 if _is_f32(A) else torch.float64
    B = CSRMatrix(np.zeros(A.numCols + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, A.dtype), A.numRows)
    B.nnz = A.nnz
    B.d_rowPtr = torch.empty(A.numCols + 1, dtype=torch.int32, device="cuda")
    B.d_colIdx = torch.empty(max(A.nnz, 1), dtype=torch.int32, device="cuda")
    B.d_values = torch.empty(max(A.nnz, 1), dtype=tdt, device="cuda")
    f = lib().spmv_csr_transpose_f32 if _is_f32(A) else lib().spmv_csr_transpose_f64
    check(f(*A.device_args(), _ptr(B.d_rowPtr), _ptr(B.d_colIdx), _ptr(B.d_values), _stream_ptr(stream)),
          "spmv_csr_transpose")
    return B


def debug_fail_allocation(n: int):
    """Tests: the n-th device allocation of the library from now fails as out
    of memory (0 turns this off); see spmv_debug_fail_allocation."""
    check(lib().spmv_debug_fail_allocation(int(n)), "spmv_debug_fail_allocation")


def debug_device_memory() -> tuple[int, int]:
    """(live bytes, live allocations) of the library's device memory."""
    b, n = C.c_longlong(), C.c_longlong()
    check(lib().spmv_debug_device_memory(C.byref(b), C.byref(n)), "spmv_debug_device_memory")
    return b.value, n.value


def make_variant(kernel: int, blockSize: int = 256, threadsPerRow: int = 0, itemsPerThread: int = 0,
                 vectorWidth: int = 1) -> Variant:
    return Variant(kernel, blockSize, threadsPerRow, itemsPerThread, vectorWidth)


def spmv_csr_variant(variant: Variant, A: CSRMatrix, x, y, alpha=1.0, beta=0.0, opts: Opts | None = None):
    o = opts if opts is not None else spmv_default_opts()
    f = lib().spmv_csr_variant_f32 if _is_f32(A) else lib().spmv_csr_variant_f64
    check(f(C.byref(variant), *A.device_args(), _ptr(x), _ptr(y), alpha, beta, C.byref(o)), "spmv_csr_variant")
    return y


def spmv_merge_based(A: CSRMatrix, x, y, stream=None):
    """spmv_merge_based<T> (src/spmv/csr5/spmv_csr5.cu:930-1014): y = A*x."""
    f = lib().spmv_merge_based_f32 if _is_f32(A) else lib().spmv_merge_based_f64
    check(f(*A.device_args(), _ptr(x), _ptr(y), _stream_ptr(stream)), "spmv_merge_based")
    return y


def merge_default_partitions(numRows: int, nnz: int) -> int:
    return lib().spmv_merge_default_partitions(numRows, nnz)


def compute_merge_partitions(numRows: int, nnz: int, numPartitions: int, stream=None):
    """compute_merge_partitions_kernel (spmv_csr5.cu:912-925) -> int32 tensor of P+1 positions."""
    torch = _torch()
    pos = torch.empty(numPartitions + 1, dtype=torch.int32, device="cuda")
    check(lib().spmv_merge_partitions(numRows, nnz, numPartitions, _ptr(pos), _stream_ptr(stream)),
          "spmv_merge_partitions")
    return pos


def merge_path_search(A: CSRMatrix, diag, stream=None):
    """merge_path_search (spmv_csr5.cu:497-533) for each diagonal in `diag` (int32 tensor)."""
    torch = _torch()
    n = diag.numel()
    r = torch.empty(n, dtype=torch.int32, device="cuda")
    z = torch.empty(n, dtype=torch.int32, device="cuda")
    check(lib().spmv_merge_path_search(_ptr(A.d_rowPtr), A.numRows, A.nnz, _ptr(diag), n, _ptr(r), _ptr(z),
                                       _stream_ptr(stream)), "spmv_merge_path_search")
    return r, z


class Plan:
    """A plan binds a device CSR matrix to one kernel variant and its
    precomputed metadata (tile coordinates, scratch)."""

    def __init__(self, handle: SpmvHandle, A: CSRMatrix, variant: Variant | None = None, copy: bool = False):
        """copy=True: the plan keeps its own copy of the matrix (SPMV_PLAN_COPY),
        so A's device arrays may be freed; otherwise it borrows them."""
        self.handle = handle
        self._f32 = _is_f32(A)
        self.A = None if copy else A  # keeps the borrowed device arrays alive
        v = variant if variant is not None else make_variant(KERNEL_AUTO)
        p = C.c_void_p()
        check(lib().spmv_plan_create_ex(handle.raw, SPMV_TYPE_FLOAT if self._f32 else SPMV_TYPE_DOUBLE,
                                        *A.device_args(), C.byref(v), 1 if copy else 0, C.byref(p)),
              "spmv_plan_create_ex")
        self._p = p

    @classmethod
    def from_format(cls, handle: SpmvHandle, A: CSRMatrix, fmt: int, params: Variant | None = None) -> "Plan":
        """spmv_convert: a plan of A in SPMV_FORMAT_CSR / _CSR5 / _ELL (borrows A)."""
        self = cls.__new__(cls)
        self.handle, self._f32, self.A = handle, _is_f32(A), A
        p = C.c_void_p()
        check(lib().spmv_convert(handle.raw, SPMV_TYPE_FLOAT if self._f32 else SPMV_TYPE_DOUBLE, *A.device_args(),
                                 int(fmt), C.byref(params) if params is not None else None, C.byref(p)),
              "spmv_convert")
        self._p = p
        return self

    @property
    def variant(self) -> Variant:
        v = Variant()
        check(lib().spmv_plan_get_variant(self._p, C.byref(v)), "spmv_plan_get_variant")
        return v

    @property
    def workspace_bytes(self) -> int:
        b = C.c_size_t()
        check(lib().spmv_plan_get_workspace_bytes(self._p, C.byref(b)), "spmv_plan_get_workspace_bytes")
        return b.value

    def exec(self, x, y, alpha=1.0, beta=0.0, transpose: bool = False):
        """y = alpha*A*x + beta*y, or alpha*A^T*x + beta*y with transpose=True
        (A^T is built on the first such call and kept)."""
        if transpose:
            f = lib().spmv_plan_exec_op_f32 if self._f32 else lib().spmv_plan_exec_op_f64
            check(f(self.handle.raw, self._p, _lib.SPMV_OP_TRANSPOSE, alpha, _ptr(x), beta, _ptr(y)),
                  "spmv_plan_exec_op")
            return y
        f = lib().spmv_plan_exec_f32 if self._f32 else lib().spmv_plan_exec_f64
        check(f(self.handle.raw, self._p, alpha, _ptr(x), beta, _ptr(y)), "spmv_plan_exec")
        return y

    def exec_op(self, op: int, x, y, alpha=1.0, beta=0.0):
        """spmv_exec_*: y = alpha*op(A)*x + beta*y, op = SPMV_OP_NORMAL / SPMV_OP_TRANSPOSE."""
        f = lib().spmv_exec_f32 if self._f32 else lib().spmv_exec_f64
        check(f(self.handle.raw, self._p, int(op), alpha, _ptr(x), beta, _ptr(y)), "spmv_exec")
        return y

    def device_error(self) -> int:
        """Device failure word of the plan (0 = clean): raised when the BAND
        kernel's bounded window wait gave up; raises SpmvError when set."""
        code = C.c_int()
        check(lib().spmv_plan_device_error(self._p, C.byref(code)), "spmv_plan_device_error")
        return code.value

    def inject_wait_timeout(self, enable: bool = True, limit_cycles: int = 0):
        """Tests: make the BAND kernel's window wait run out (see
        spmv_plan_inject_wait_timeout)."""
        check(lib().spmv_plan_inject_wait_timeout(self._p, 1 if enable else 0, int(limit_cycles)),
              "spmv_plan_inject_wait_timeout")

    def profile(self, enable: bool = True):
        """Records CUDA events around the main kernel of every exec."""
        check(lib().spmv_plan_profile(self._p, 1 if enable else 0), "spmv_plan_profile")

    def profile_read(self):
        """(summed main-kernel milliseconds, launches) since profile() / the last read."""
        ms, n = C.c_double(), C.c_int()
        check(lib().spmv_plan_profile_read(self._p, C.byref(ms), C.byref(n)), "spmv_plan_profile_read")
        return ms.value, n.value

    def destroy(self):
        if self._p:
            check(lib().spmv_plan_destroy(self._p), "spmv_plan_destroy")
            self._p = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Pipeline:
    """Host-to-host SpMV: x from pinned host memory, y to pinned host memory,
    copies overlapped with the SpMV (row slices copied out as they finish,
    `depth` requests in flight).  The pinned-memory / multi-stream path of the
    reference's tests/test_pinned_memory.cu:245-380."""

    def __init__(self, handle: SpmvHandle, A: CSRMatrix, variant: Variant | None = None, slices: int = 0,
                 depth: int = 0):
        self.handle = handle
        self.A = A
        p = C.c_void_p()
        check(lib().spmv_pipeline_create(handle.raw, SPMV_TYPE_FLOAT if _is_f32(A) else SPMV_TYPE_DOUBLE,
                                         *A.device_args(), C.byref(variant) if variant is not None else None,
                                         slices, depth, C.byref(p)), "spmv_pipeline_create")
        self._p = p
        self._held = []  # host tensors of requests in flight

    def info(self) -> dict:
        sl, dp, lp = C.c_int(), C.c_int(), C.c_int()
        v, b = Variant(), C.c_size_t()
        check(lib().spmv_pipeline_info(self._p, C.byref(sl), C.byref(dp), C.byref(v), C.byref(b), C.byref(lp)),
              "spmv_pipeline_info")
        return {"slices": sl.value, "depth": dp.value, "variant": v.as_dict(), "device_bytes": b.value,
                "launches_per_request": lp.value}

    def submit(self, hx, hy, alpha=1.0, beta=0.0):
        """Enqueues y = alpha*A*x + beta*y for host tensors hx, hy (pinned for
        overlap); hy is complete after wait()."""
        f = lib().spmv_pipeline_submit_f32 if _is_f32(self.A) else lib().spmv_pipeline_submit_f64
        check(f(self._p, alpha, _ptr(hx), beta, _ptr(hy)), "spmv_pipeline_submit")
        self._held.append((hx, hy))
        return hy

    def wait(self):
        check(lib().spmv_pipeline_wait(self._p), "spmv_pipeline_wait")
        self._held.clear()

    def order_after(self, stream):
        check(lib().spmv_pipeline_order_after(self._p, _stream_ptr(stream)), "spmv_pipeline_order_after")

    def join(self, stream):
        check(lib().spmv_pipeline_join(self._p, _stream_ptr(stream)), "spmv_pipeline_join")

    def destroy(self):
        if self._p:
            check(lib().spmv_pipeline_destroy(self._p), "spmv_pipeline_destroy")
            self._p = None
            self._held.clear()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# CSR5 (src/spmv/csr5/spmv_csr5.cuh, src/formats/sparse_formats.h:284-386)
# ---------------------------------------------------------------------------
class CSR5Matrix:
    """CSR5Matrix<T>: borrows the CSR arrays (referenceFromCSR) and owns the
    tile metadata d_tile_row_ptr / d_tile_nnz_offset (torch int32)."""

    def __init__(self, csr: CSRMatrix):
        self.csr = csr
        self.numRows, self.numCols, self.nnz = csr.numRows, csr.numCols, csr.nnz
        self.sigma = 0
        self.numTiles = 0
        self.d_tile_row_ptr = self.d_tile_nnz_offset = None


def csr5_preprocess(csr: CSRMatrix, csr5: CSR5Matrix | None = None, sigma: int = 0, stream=None) -> CSR5Matrix:
    """csr5_preprocess<T> (spmv_csr5.cu:223-275); sigma <= 0 picks the warp-32 default (128)."""
    torch = _torch()
    m = csr5 if csr5 is not None else CSR5Matrix(csr)
    m.sigma = sigma if sigma > 0 else lib().spmv_csr5_default_sigma()
    m.numTiles = lib().spmv_csr5_num_tiles(csr.nnz, m.sigma)
    m.d_tile_row_ptr = torch.empty(max(m.numTiles, 1), dtype=torch.int32, device="cuda")
    m.d_tile_nnz_offset = torch.empty(max(m.numTiles, 1), dtype=torch.int32, device="cuda")
    check(lib().spmv_csr5_preprocess(_ptr(csr.d_rowPtr), csr.numRows, csr.nnz, m.sigma, _ptr(m.d_tile_row_ptr),
                                     _ptr(m.d_tile_nnz_offset), _stream_ptr(stream)), "csr5_preprocess")
    return m


def spmv_csr5(m: CSR5Matrix, x, y, alpha=1.0, beta=0.0, opts: Opts | None = None):
    """spmv_csr5<T> (spmv_csr5.cu:277-362) with alpha/beta applied."""
    o = opts if opts is not None else spmv_default_opts()
    A = m.csr
    f = lib().spmv_csr5_f32 if _is_f32(A) else lib().spmv_csr5_f64
    check(f(*A.device_args(), m.sigma, _ptr(m.d_tile_row_ptr), _ptr(m.d_tile_nnz_offset), _ptr(x), _ptr(y), alpha,
            beta, C.byref(o)), "spmv_csr5")
    return y


# ---------------------------------------------------------------------------
# ELLPACK (src/spmv/ellpack/spmv_ellpack.cuh:26-39)
# ---------------------------------------------------------------------------
class ELLPACKMatrix:
    def __init__(self):
        self.numRows = self.numCols = self.numElements = self.nnz = 0
        self.d_colIdx = self.d_values = None
        self.truncatedRows = 0


def max_row_length(A: CSRMatrix, stream=None) -> int:
    w = C.c_int()
    check(lib().spmv_max_row_length(_ptr(A.d_rowPtr), A.numRows, C.byref(w), _stream_ptr(stream)), "max_row_length")
    return w.value


def csr_to_ellpack(A: CSRMatrix, ell: ELLPACKMatrix | None = None, maxElements: int = 0, stream=None):
    """csr_to_ellpack<T> (spmv_ellpack.cu:11-70) on the GPU; maxElements <= 0 = longest row."""
    torch = _torch()
    e = ell if ell is not None else ELLPACKMatrix()
    W = maxElements if maxElements > 0 else max_row_length(A, stream)
    e.numRows, e.numCols, e.numElements, e.nnz = A.numRows, A.numCols, W, A.nnz
    tdt = torch.float32 if _is_f32(A) else torch.float64
    e.d_colIdx = torch.empty(max(A.numRows * W, 1), dtype=torch.int32, device="cuda")
    e.d_values = torch.empty(max(A.numRows * W, 1), dtype=tdt, device="cuda")
    t = C.c_longlong()
    f = lib().spmv_csr_to_ell_f32 if _is_f32(A) else lib().spmv_csr_to_ell_f64
    check(f(A.numRows, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(A.d_values), W, _ptr(e.d_colIdx),
            _ptr(e.d_values), C.byref(t), _stream_ptr(stream)), "csr_to_ellpack")
    e.truncatedRows = t.value
    return e


def spmv_ellpack(e: ELLPACKMatrix, x, y, stream=None, alpha=1.0, beta=0.0):
    """spmv_ellpack<T> (spmv_ellpack.cu:72-91)."""
    f = lib().spmv_ellpack_f32 if e.d_values.dtype == _torch().float32 else lib().spmv_ellpack_f64
    check(f(e.numRows, e.numElements, _ptr(e.d_colIdx), _ptr(e.d_values), _ptr(x), _ptr(y), alpha, beta,
            _stream_ptr(stream)), "spmv_ellpack")
    return y


# ---------------------------------------------------------------------------
# Reorders
# ---------------------------------------------------------------------------
COLPERM_CENTER_OF_MASS, COLPERM_MIN_ROW, COLPERM_FREQUENCY = 0, 1, 2


def reorder_rows_by_length(A: CSRMatrix, stream=None):
    """reorderMatrixByRowLength (tests/test_row_reordering.cu:99-143) on the
    GPU: returns (rowMap, reordered CSRMatrix with device arrays)."""
    torch = _torch()
    rm = torch.empty(max(A.numRows, 1), dtype=torch.int32, device="cuda")
    B = CSRMatrix(A.rowPtr, A.colIdx, A.values, A.numCols)
    B.allocateDevice()
    f = lib().spmv_reorder_rows_by_length_f32 if _is_f32(A) else lib().spmv_reorder_rows_by_length_f64
    check(f(A.numRows, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(A.d_values), _ptr(rm), _ptr(B.d_rowPtr),
            _ptr(B.d_colIdx), _ptr(B.d_values), _stream_ptr(stream)), "reorder_rows_by_length")
    return rm[: A.numRows], B


def restore_order(y_perm, rowMap, y, stream=None):
    f = lib().spmv_restore_order_f32 if y.dtype == _torch().float32 else lib().spmv_restore_order_f64
    check(f(y.numel(), _ptr(y_perm), _ptr(rowMap), _ptr(y), _stream_ptr(stream)), "restore_order")
    return y


def column_perm(A: CSRMatrix, kind: int, stream=None):
    """(perm new->old, keys) for a column order (see spmv_colperm_t)."""
    torch = _torch()
    perm = torch.empty(max(A.numCols, 1), dtype=torch.int32, device="cuda")
    kdt = torch.float32 if kind == COLPERM_CENTER_OF_MASS else torch.int32
    keys = torch.empty(max(A.numCols, 1), dtype=kdt, device="cuda")
    check(lib().spmv_column_perm(kind, A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(perm),
                                 _ptr(keys), _stream_ptr(stream)), "column_perm")
    return perm[: A.numCols], keys[: A.numCols]


def apply_column_perm(A: CSRMatrix, perm, stream=None):
    torch = _torch()
    out = torch.empty(max(A.nnz, 1), dtype=torch.int32, device="cuda")
    check(lib().spmv_apply_column_perm(A.numCols, A.nnz, _ptr(perm), _ptr(A.d_colIdx), _ptr(out),
                                       _stream_ptr(stream)), "apply_column_perm")
    return out[: A.nnz]


def permute_x(perm, x, stream=None):
    xr = _torch().empty_like(x)
    f = lib().spmv_permute_x_f32 if x.dtype == _torch().float32 else lib().spmv_permute_x_f64
    check(f(x.numel(), _ptr(perm), _ptr(x), _ptr(xr), _stream_ptr(stream)), "permute_x")
    return xr


def sort_columns_within_rows(A: CSRMatrix, stream=None):
    """sortColumnsWithinRows (column_reorder.cuh:175-201), in place on A's device arrays."""
    f = lib().spmv_sort_columns_within_rows_f32 if _is_f32(A) else lib().spmv_sort_columns_within_rows_f64
    check(f(A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), _ptr(A.d_values), _stream_ptr(stream)),
          "sort_columns_within_rows")
    return A


def count_distinct_columns(A: CSRMatrix, stream=None) -> int:
    d = C.c_longlong()
    check(lib().spmv_count_distinct_columns(A.numCols, A.nnz, _ptr(A.d_colIdx), C.byref(d), _stream_ptr(stream)),
          "spmv_count_distinct_columns")
    return d.value


def validate_csr(A: CSRMatrix, stream=None) -> int:
    b = C.c_longlong()
    check(lib().spmv_validate_csr(A.numRows, A.numCols, A.nnz, _ptr(A.d_rowPtr), _ptr(A.d_colIdx), C.byref(b),
                                  _stream_ptr(stream)), "spmv_validate_csr")
    return b.value


# ---------------------------------------------------------------------------
# Matrix Market I/O (src/generators/mtx_io.h:22-85)
# ---------------------------------------------------------------------------
def readMTXHeader(filename) -> dict:
    h = _lib.MtxHeader()
    check(lib().spmv_mtx_read_header(str(filename).encode(), C.byref(h)), "spmv_mtx_read_header")
    return {k: getattr(h, k) for k, _ in h._fields_}


def readMTXFile(filename, dtype=np.float32, expandSymmetric: bool = True) -> CSRMatrix:
    """readMTXFile<T> (mtx_io.cu:111-222) -> CSRMatrix with host arrays."""
    h = _lib.HostCSR()
    t = SPMV_TYPE_FLOAT if np.dtype(dtype) == np.float32 else SPMV_TYPE_DOUBLE
    check(lib().spmv_mtx_read(str(filename).encode(), t, 1 if expandSymmetric else 0, C.byref(h)), "spmv_mtx_read")
    try:
        rp = np.ctypeslib.as_array(h.rowPtr, shape=(h.numRows + 1,)).copy()
        ci = np.ctypeslib.as_array(h.colIdx, shape=(max(h.nnz, 1),))[:h.nnz].copy()
        vt = C.c_float if t == SPMV_TYPE_FLOAT else C.c_double
        va = np.ctypeslib.as_array(C.cast(h.values, C.POINTER(vt)), shape=(max(h.nnz, 1),))[:h.nnz].copy()
    finally:
        lib().spmv_host_csr_free(C.byref(h))
    return CSRMatrix(rp, ci, va, h.numCols)


def writeMTXFile(filename, A: CSRMatrix, writeSymmetric: bool = False):
    """writeMTXFile<T> (mtx_io.cu:224-271), banner fixed, exact values."""
    rp = np.ascontiguousarray(A.rowPtr, np.int32)
    ci = np.ascontiguousarray(A.colIdx, np.int32)
    va = np.ascontiguousarray(A.values)
    h = _lib.HostCSR(A.numRows, A.numCols, A.nnz, rp.ctypes.data_as(C.POINTER(C.c_int)),
                     ci.ctypes.data_as(C.POINTER(C.c_int)), va.ctypes.data_as(C.c_void_p),
                     SPMV_TYPE_FLOAT if va.dtype == np.float32 else SPMV_TYPE_DOUBLE)
    check(lib().spmv_mtx_write(str(filename).encode(), C.byref(h), 1 if writeSymmetric else 0), "spmv_mtx_write")


# ---------------------------------------------------------------------------
# Generators (host)
# ---------------------------------------------------------------------------
GEN_POISSON_UNIFORM, GEN_POWERLAW, GEN_STENCIL2D, GEN_STENCIL3D, GEN_BANDED, GEN_BLOCKDIAG, GEN_ZIPF_UNIFORM, \
    GEN_DIAGONAL = range(8)


@dataclass
class GenSpec:
    kind: int
    numRows: int
    numCols: int
    p0: float = 0.0
    p1: float = 0.0
    p2: float = 0.0
    p3: float = 0.0
    seed: int = 0

    def params(self, threads: int = 0) -> GenParams:
        return GenParams(self.kind, self.numRows, self.numCols, self.p0, self.p1, self.p2, self.p3, self.seed,
                         threads)


def generate(spec: GenSpec, dtype=np.float32, threads: int = 0, pinned: bool = False):
    """Returns host (rowPtr, colIdx, values) numpy arrays for `spec`.
    pinned=True places the arrays in page-locked memory (torch)."""
    p = spec.params(threads)
    rowPtr = np.empty(spec.numRows + 1, np.int32)
    nnz = C.c_longlong()
    check(lib().spmv_gen_row_ptr(C.byref(p), rowPtr.ctypes.data_as(C.c_void_p), C.byref(nnz)), "spmv_gen_row_ptr")
    n = nnz.value
    if pinned:
        torch = _torch()
        tdt = torch.float32 if dtype == np.float32 else torch.float64
        colIdx = torch.empty(max(n, 1), dtype=torch.int32, pin_memory=True).numpy()[:n]
        values = torch.empty(max(n, 1), dtype=tdt, pin_memory=True).numpy()[:n]
    else:
        colIdx = np.empty(n, np.int32)
        values = np.empty(n, dtype)
    f = lib().spmv_gen_fill_f32 if dtype == np.float32 else lib().spmv_gen_fill_f64
    check(f(C.byref(p), rowPtr.ctypes.data_as(C.c_void_p), colIdx.ctypes.data_as(C.c_void_p),
            values.ctypes.data_as(C.c_void_p)), "spmv_gen_fill")
    return rowPtr, colIdx, values


def gen_vector(n: int, seed: int, lo: float = -1.0, hi: float = 1.0, dtype=np.float32, threads: int = 0, out=None):
    v = out if out is not None else np.empty(n, dtype)
    f = lib().spmv_gen_vector_f32 if v.dtype == np.float32 else lib().spmv_gen_vector_f64
    check(f(n, seed, lo, hi, v.ctypes.data_as(C.c_void_p), threads), "spmv_gen_vector")
    return v


__all__ = [n for n in dir() if not n.startswith("_")]
