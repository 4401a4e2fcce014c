"""ctypes binding of libmuxispmv.so (the C ABI declared in include/muxi_spmv.h).

The shared library is built in-tree by muxi_spmv_gb300.build.  Loading fails
loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

LIB_PATH = _build.LIB

# Status codes (src/utils/common.h:31-43).
SPMV_SUCCESS = 0
STATUS_NAMES = {
    0: "SPMV_SUCCESS", -1: "SPMV_ERROR_INVALID_HANDLE", -2: "SPMV_ERROR_INVALID_MATRIX",
    -3: "SPMV_ERROR_INVALID_VECTOR", -4: "SPMV_ERROR_MEMORY_ALLOC", -5: "SPMV_ERROR_MEMORY_COPY",
    -6: "SPMV_ERROR_DEVICE", -7: "SPMV_ERROR_UNSUPPORTED_FORMAT", -8: "SPMV_ERROR_UNSUPPORTED_TYPE",
    -9: "SPMV_ERROR_INTERNAL",
}

SPMV_TYPE_FLOAT, SPMV_TYPE_DOUBLE = 0, 1
SPMV_OP_NORMAL, SPMV_OP_TRANSPOSE = 0, 1
SPMV_FORMAT_CSR, SPMV_FORMAT_COO, SPMV_FORMAT_CSR2, SPMV_FORMAT_BSR, SPMV_FORMAT_CSR5, SPMV_FORMAT_ELL = 0, 1, 2, 3, 4, 5

KERNEL_AUTO, KERNEL_SCALAR, KERNEL_VECTOR, KERNEL_MERGE, KERNEL_CSR5, KERNEL_ELL, KERNEL_HEURISTIC, \
    KERNEL_BAND, KERNEL_STREAM = range(9)
CSR5_ORDERED, CSR5_ORDERED_PREFETCH = 32, 64
RANGE_PER_RESIDENT_BLOCK = 1 << 20


class SpmvError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} ({status}): {detail}")


class Opts(C.Structure):
    """spmv_opts_t (src/utils/common.h:73-82)."""
    _fields_ = [("operation", C.c_int), ("sync", C.c_int), ("check_inputs", C.c_int),
                ("use_tensor_core", C.c_int), ("use_streaming", C.c_int), ("stream_id", C.c_int),
                ("stream", C.c_void_p)]


class Handle(C.Structure):
    """spmv_handle_t (src/api/spmv_api.h:18-28 plus GB300 fields)."""
    _fields_ = [("deviceId", C.c_int), ("stream", C.c_void_p), ("opts", Opts), ("warpSize", C.c_int),
                ("smCount", C.c_int), ("maxThreadsPerBlock", C.c_int), ("sharedMemPerSM", C.c_size_t),
                ("l2CacheBytes", C.c_size_t), ("sharedMemPerBlockOptin", C.c_size_t), ("ccMajor", C.c_int),
                ("ccMinor", C.c_int), ("internal", C.c_void_p)]


class Variant(C.Structure):
    """spmv_variant_t."""
    _fields_ = [("kernel", C.c_int), ("blockSize", C.c_int), ("threadsPerRow", C.c_int),
                ("itemsPerThread", C.c_int), ("vectorWidth", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GenParams(C.Structure):
    """spmv_gen_params_t."""
    _fields_ = [("kind", C.c_int), ("numRows", C.c_int), ("numCols", C.c_int), ("p0", C.c_double),
                ("p1", C.c_double), ("p2", C.c_double), ("p3", C.c_double), ("seed", C.c_ulonglong),
                ("threads", C.c_int)]


class BatchMatrix(C.Structure):
    """spmv_batch_matrix_t."""
    _fields_ = [("numRows", C.c_int), ("numCols", C.c_int), ("nnz", C.c_int), ("rowPtr", C.c_void_p),
                ("colIdx", C.c_void_p), ("values", C.c_void_p)]


class MtxHeader(C.Structure):
    """spmv_mtx_header_t."""
    _fields_ = [("isSymmetric", C.c_int), ("isSkew", C.c_int), ("isComplex", C.c_int), ("isPattern", C.c_int),
                ("isInteger", C.c_int), ("numRows", C.c_int), ("numCols", C.c_int), ("nnz", C.c_int)]


class HostCSR(C.Structure):
    """spmv_host_csr_t."""
    _fields_ = [("numRows", C.c_int), ("numCols", C.c_int), ("nnz", C.c_int), ("rowPtr", C.POINTER(C.c_int)),
                ("colIdx", C.POINTER(C.c_int)), ("values", C.c_void_p), ("type", C.c_int)]


class BatchVariant(C.Structure):
    """spmv_batch_variant_t."""
    _fields_ = [("nnzPerSlot", C.c_int), ("blocksPerSM", C.c_int), ("chunkNnz", C.c_int), ("ordered", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
I = C.c_int
F = C.c_float
D = C.c_double
S = C.c_int  # spmv_status_t

# name -> (restype, argtypes)
SIGNATURES = {
    "spmv_default_opts": (Opts, []),
    "spmv_create_handle": (S, [C.POINTER(C.POINTER(Handle))]),
    "spmv_destroy_handle": (S, [C.POINTER(Handle)]),
    "spmv_set_stream": (S, [C.POINTER(Handle), P]),
    "spmv_last_error": (C.c_char_p, []),
    "spmv_abi_version": (I, []),
    "spmv_csr_f32": (S, [I, I, I, P, P, P, P, P, F, F, C.POINTER(Opts)]),
    "spmv_csr_f64": (S, [I, I, I, P, P, P, P, P, D, D, C.POINTER(Opts)]),
    "spmv_csr_noalloc_f32": (S, [I, I, I, P, P, P, P, P, F, F, P]),
    "spmv_csr_variant_f32": (S, [C.POINTER(Variant), I, I, I, P, P, P, P, P, F, F, C.POINTER(Opts)]),
    "spmv_csr_variant_f64": (S, [C.POINTER(Variant), I, I, I, P, P, P, P, P, D, D, C.POINTER(Opts)]),
    "spmv_merge_default_partitions": (I, [I, I]),
    "spmv_merge_partitions": (S, [I, I, I, P, P]),
    "spmv_merge_path_search": (S, [P, I, I, P, I, P, P, P]),
    "spmv_merge_based_f32": (S, [I, I, I, P, P, P, P, P, P]),
    "spmv_merge_based_f64": (S, [I, I, I, P, P, P, P, P, P]),
    "spmv_csr5_default_sigma": (I, []),
    "spmv_csr5_num_tiles": (I, [I, I]),
    "spmv_csr5_preprocess": (S, [P, I, I, I, P, P, P]),
    "spmv_csr5_f32": (S, [I, I, I, P, P, P, I, P, P, P, P, F, F, C.POINTER(Opts)]),
    "spmv_csr5_f64": (S, [I, I, I, P, P, P, I, P, P, P, P, D, D, C.POINTER(Opts)]),
    "spmv_max_row_length": (S, [P, I, C.POINTER(C.c_int), P]),
    "spmv_csr_to_ell_f32": (S, [I, I, P, P, P, I, P, P, C.POINTER(C.c_longlong), P]),
    "spmv_csr_to_ell_f64": (S, [I, I, P, P, P, I, P, P, C.POINTER(C.c_longlong), P]),
    "spmv_ellpack_f32": (S, [I, I, P, P, P, P, F, F, P]),
    "spmv_ellpack_f64": (S, [I, I, P, P, P, P, D, D, P]),
    "spmv_reorder_rows_by_length_f32": (S, [I, I, P, P, P, P, P, P, P, P]),
    "spmv_reorder_rows_by_length_f64": (S, [I, I, P, P, P, P, P, P, P, P]),
    "spmv_restore_order_f32": (S, [I, P, P, P, P]),
    "spmv_restore_order_f64": (S, [I, P, P, P, P]),
    "spmv_column_perm": (S, [I, I, I, I, P, P, P, P, P]),
    "spmv_apply_column_perm": (S, [I, I, P, P, P, P]),
    "spmv_permute_x_f32": (S, [I, P, P, P, P]),
    "spmv_permute_x_f64": (S, [I, P, P, P, P]),
    "spmv_sort_columns_within_rows_f32": (S, [I, I, I, P, P, P, P]),
    "spmv_sort_columns_within_rows_f64": (S, [I, I, I, P, P, P, P]),
    "spmv_plan_create": (S, [C.POINTER(Handle), I, I, I, I, P, P, P, C.POINTER(Variant), C.POINTER(P)]),
    "spmv_plan_destroy": (S, [P]),
    "spmv_plan_create_ex": (S, [C.POINTER(Handle), I, I, I, I, P, P, P, C.POINTER(Variant), I, C.POINTER(P)]),
    "spmv_plan_get_variant": (S, [P, C.POINTER(Variant)]),
    "spmv_plan_get_workspace_bytes": (S, [P, C.POINTER(C.c_size_t)]),
    "spmv_plan_exec_f32": (S, [C.POINTER(Handle), P, F, P, F, P]),
    "spmv_plan_exec_f64": (S, [C.POINTER(Handle), P, D, P, D, P]),
    "spmv_plan_exec_op_f32": (S, [C.POINTER(Handle), P, I, F, P, F, P]),
    "spmv_convert": (S, [C.POINTER(Handle), I, I, I, I, P, P, P, I, C.POINTER(Variant), C.POINTER(P)]),
    "spmv_exec_f32": (S, [C.POINTER(Handle), P, I, F, P, F, P]),
    "spmv_exec_f64": (S, [C.POINTER(Handle), P, I, D, P, D, P]),
    "spmv_plan_exec_op_f64": (S, [C.POINTER(Handle), P, I, D, P, D, P]),
    "spmv_plan_device_error": (S, [P, C.POINTER(C.c_int)]),
    "spmv_plan_inject_wait_timeout": (S, [P, I, C.c_longlong]),
    "spmv_debug_fail_allocation": (S, [C.c_longlong]),
    "spmv_debug_device_memory": (S, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "spmv_plan_profile": (S, [P, I]),
    "spmv_plan_profile_read": (S, [P, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "spmv_count_distinct_columns": (S, [I, I, P, C.POINTER(C.c_longlong), P]),
    "spmv_validate_csr": (S, [I, I, I, P, P, C.POINTER(C.c_longlong), P]),
    "spmv_gen_row_ptr": (S, [C.POINTER(GenParams), P, C.POINTER(C.c_longlong)]),
    "spmv_gen_fill_f32": (S, [C.POINTER(GenParams), P, P, P]),
    "spmv_gen_fill_f64": (S, [C.POINTER(GenParams), P, P, P]),
    "spmv_gen_vector_f32": (S, [C.c_longlong, C.c_ulonglong, D, D, P, I]),
    "spmv_gen_vector_f64": (S, [C.c_longlong, C.c_ulonglong, D, D, P, I]),
    "spmv_gen_device_row_ptr": (S, [C.POINTER(GenParams), P, C.POINTER(C.c_longlong), P]),
    "spmv_gen_device_fill_f32": (S, [C.POINTER(GenParams), P, P, P, P]),
    "spmv_gen_device_vector_f32": (S, [C.c_longlong, C.c_ulonglong, D, D, P, P]),
    "spmv_matrix_features": (S, [I, I, I, I, P, P, P, P]),
    "spmv_variant_space": (I, [P, I]),
    "spmv_autotune": (S, [C.POINTER(Handle), I, I, I, I, P, P, P, P, I, I, P, C.POINTER(C.c_int)]),
    "spmv_mlp_create": (S, [I, I, I, I, C.c_ulonglong, C.POINTER(P)]),
    "spmv_mlp_destroy": (S, [P]),
    "spmv_mlp_num_params": (I, [P]),
    "spmv_mlp_shape": (S, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "spmv_mlp_get_params": (S, [P, P, I]),
    "spmv_mlp_set_params": (S, [P, P, I]),
    "spmv_mlp_set_normalization": (S, [P, P, P]),
    "spmv_mlp_forward": (S, [P, P, P, I, P]),
    "spmv_mlp_gradients": (S, [P, P, P, P, I, C.POINTER(F), P, P]),
    "spmv_mlp_train_step": (S, [P, P, P, P, I, F, C.POINTER(F), P]),
    "spmv_mlp_save": (S, [P, C.c_char_p]),
    "spmv_mlp_load": (S, [C.c_char_p, C.POINTER(P)]),
    "spmv_select": (S, [C.POINTER(Handle), I, P, I, I, I, I, I, P, P, P, C.POINTER(Variant), C.POINTER(C.c_int)]),
    "spmv_set_selector": (S, [C.POINTER(Handle), P]),
    "spmv_csr_transpose_f32": (S, [I, I, I, P, P, P, P, P, P, P]),
    "spmv_csr_transpose_f64": (S, [I, I, I, P, P, P, P, P, P, P]),
    "spmv_mtx_read_header": (S, [C.c_char_p, C.POINTER(MtxHeader)]),
    "spmv_mtx_read": (S, [C.c_char_p, I, I, C.POINTER(HostCSR)]),
    "spmv_mtx_write": (S, [C.c_char_p, C.POINTER(HostCSR), I]),
    "spmv_host_csr_free": (None, [C.POINTER(HostCSR)]),
    "spmv_batch_create": (S, [C.POINTER(Handle), I, C.POINTER(BatchMatrix), I, C.POINTER(P)]),
    "spmv_batch_create_ex": (S, [C.POINTER(Handle), I, C.POINTER(BatchMatrix), I, C.POINTER(BatchVariant),
                                 C.POINTER(P)]),
    "spmv_batch_get_variant": (S, [P, C.POINTER(BatchVariant)]),
    "spmv_batch_destroy": (S, [P]),
    "spmv_batch_set_vectors_f32": (S, [P, C.POINTER(P), C.POINTER(P)]),
    "spmv_batch_exec_f32": (S, [C.POINTER(Handle), P, F, F, I]),
    "spmv_batch_info": (S, [P, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "spmv_batch_group_create": (S, [C.POINTER(Handle), I, C.POINTER(BatchMatrix), C.POINTER(C.c_int),
                                    C.POINTER(BatchVariant), C.POINTER(P)]),
    "spmv_batch_group_destroy": (S, [P]),
    "spmv_batch_group_set_vectors_f32": (S, [P, P, P]),
    "spmv_batch_group_exec_f32": (S, [C.POINTER(Handle), P, F, F, I]),
    "spmv_batch_group_info": (S, [P, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "spmv_set_selector_mode": (S, [C.POINTER(Handle), I]),
    "spmv_csr_to_bsr_count": (S, [I, I, I, P, P, I, P, C.POINTER(C.c_int), P]),
    "spmv_csr_to_bsr_f32": (S, [I, I, I, P, P, P, I, P, P, P, P]),
    "spmv_csr_to_bsr_f64": (S, [I, I, I, P, P, P, I, P, P, P, P]),
    "spmv_bsr_f32": (S, [I, I, I, I, P, P, P, P, P, F, F, P]),
    "spmv_bsr_f64": (S, [I, I, I, I, P, P, P, P, P, D, D, P]),
    "spmv_coo_to_csr_f32": (S, [I, I, I, P, P, P, P, P, P, P]),
    "spmv_coo_to_csr_f64": (S, [I, I, I, P, P, P, P, P, P, P]),
    "spmv_coo_f32": (S, [I, I, I, P, P, P, P, P, F, F, C.POINTER(Opts)]),
    "spmv_coo_f64": (S, [I, I, I, P, P, P, P, P, D, D, C.POINTER(Opts)]),
    "spmv_pipeline_create": (S, [C.POINTER(Handle), I, I, I, I, P, P, P, C.POINTER(Variant), I, I, C.POINTER(P)]),
    "spmv_pipeline_destroy": (S, [P]),
    "spmv_pipeline_submit_f32": (S, [P, F, P, F, P]),
    "spmv_pipeline_submit_f64": (S, [P, D, P, D, P]),
    "spmv_pipeline_wait": (S, [P]),
    "spmv_pipeline_order_after": (S, [P, P]),
    "spmv_pipeline_join": (S, [P, P]),
    "spmv_pipeline_info": (S, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(Variant),
                               C.POINTER(C.c_size_t), C.POINTER(C.c_int)]),
}

BATCH_PERSISTENT, BATCH_PERSISTENT_GRAPH, BATCH_LOOP, BATCH_LOOP_GRAPH = range(4)

NUM_FEATURES = 32
SELECT_HEURISTIC, SELECT_LEARNED, SELECT_AUTOTUNE, SELECT_LEARNED_TOPK, SELECT_LEARNED_FALLBACK = range(5)
FALLBACK_MARGIN = 0.12  # predicted log-time gap of SELECT_LEARNED_FALLBACK (select.cu)
FALLBACK_MAX = 4  # candidates it times at most, the pick included (select.cu)

_lib = None


def lib() -> C.CDLL:
    """Loads (building if needed) libmuxispmv.so and declares every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if os.environ.get("MUXI_SPMV_NO_BUILD"):
            raise ImportError(f"{LIB_PATH} is missing; run __graft_entry__.build() first")
        _build.build()
    L = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return (lib().spmv_last_error() or b"").decode(errors="replace")


def check(status: int, where: str) -> None:
    if status != SPMV_SUCCESS:
        raise SpmvError(status, where, last_error())
