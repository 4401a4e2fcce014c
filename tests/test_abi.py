"""The C ABI boundary on a CPU-only machine: the library loads, exports every
entry point include/*.h declares, the header compiles as C, enum values equal
the reference's (src/utils/common.h:31-70), argument validation returns the
reference's status codes without touching a device, and the host generators
are deterministic."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        for m in re.finditer(r"^SPMV_API\s+[^;(]*?\b(spmv_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(mx):
    lib = mx.lib()
    names = declared_symbols()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(mx._lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert set(names) <= exported
    # nothing but the declared entry points leaks out of the library
    assert {e for e in exported if e.startswith("spmv_")} == set(names)


def test_python_binding_covers_the_header(mx):
    assert set(declared_symbols()) == set(mx._lib.SIGNATURES)


def test_header_is_plain_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text(r'''
#include "muxi_spmv.h"
_Static_assert(SPMV_SUCCESS == 0 && SPMV_ERROR_INVALID_HANDLE == -1 && SPMV_ERROR_INVALID_MATRIX == -2, "st");
_Static_assert(SPMV_ERROR_INVALID_VECTOR == -3 && SPMV_ERROR_MEMORY_ALLOC == -4 && SPMV_ERROR_MEMORY_COPY == -5, "st");
_Static_assert(SPMV_ERROR_DEVICE == -6 && SPMV_ERROR_UNSUPPORTED_FORMAT == -7, "st");
_Static_assert(SPMV_ERROR_UNSUPPORTED_TYPE == -8 && SPMV_ERROR_INTERNAL == -9, "st");
_Static_assert(SPMV_FORMAT_CSR == 0 && SPMV_FORMAT_COO == 1 && SPMV_FORMAT_CSR2 == 2 && SPMV_FORMAT_BSR == 3, "fmt");
_Static_assert(SPMV_FORMAT_CSR5 == 4 && SPMV_FORMAT_UNKNOWN == -1, "fmt");
_Static_assert(SPMV_TYPE_FLOAT == 0 && SPMV_TYPE_DOUBLE == 1 && SPMV_TYPE_HALF == 2 && SPMV_TYPE_BF16 == 3, "ty");
_Static_assert(SPMV_TYPE_TF32 == 4 && SPMV_TYPE_UNKNOWN == -1, "ty");
_Static_assert(SPMV_OP_NORMAL == 0 && SPMV_OP_TRANSPOSE == 1 && SPMV_OP_CONJUGATE == 2, "op");
int main(void) { spmv_opts_t o = spmv_default_opts(); return o.sync; }
''')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-c", "-I", str(ROOT / "include"), "-I",
                        "/usr/local/cuda/include", str(src), "-o", str(tmp_path / "t.o")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr


def test_default_opts(mx):
    o = mx.lib().spmv_default_opts()
    assert (o.operation, o.sync, o.check_inputs, o.use_tensor_core, o.use_streaming, o.stream_id) == (0, 0, 0, 0, 0, 0)
    assert o.stream is None
    assert mx.lib().spmv_abi_version() == 1


def test_argument_errors_without_device(mx):
    """Validation happens before any device work and returns the reference's
    status codes; the message names the problem."""
    L = mx.lib()
    o = L.spmv_default_opts()
    import ctypes as C
    st = L.spmv_csr_f32(-1, 4, 0, None, None, None, None, None, 1.0, 0.0, C.byref(o))
    assert st == -2 and "negative" in mx.last_error()
    st = L.spmv_csr_f32(4, 4, 3, None, None, None, None, None, 1.0, 0.0, C.byref(o))
    assert st == -2 and "rowPtr" in mx.last_error()
    st = L.spmv_destroy_handle(None)
    assert st == -1
    st = L.spmv_merge_partitions(10, 10, 0, None, None)
    assert st == -2
    o.operation = 2  # conjugate: real types only
    st = L.spmv_csr_f32(4, 4, 0, 1, None, None, None, 1, 1.0, 0.0, C.byref(o))
    assert st == -7
    o.operation = 1  # transpose: argument checks come before any device work
    st = L.spmv_csr_f32(4, 4, 3, None, None, None, None, None, 1.0, 0.0, C.byref(o))
    assert st == -2 and "rowPtr" in mx.last_error()
    # the format-generic pair: formats without a plan, missing handle / plan
    p = C.c_void_p()
    for fmt in (mx.SPMV_FORMAT_COO, mx.SPMV_FORMAT_CSR2, mx.SPMV_FORMAT_BSR, -1):
        st = L.spmv_convert(None, mx.SPMV_TYPE_FLOAT, 4, 4, 0, None, None, None, fmt, None, C.byref(p))
        assert st == -7 and "CSR, CSR5 or ELL" in mx.last_error()
    for fmt in (mx.SPMV_FORMAT_CSR, mx.SPMV_FORMAT_CSR5, mx.SPMV_FORMAT_ELL):
        st = L.spmv_convert(None, mx.SPMV_TYPE_FLOAT, 4, 4, 0, None, None, None, fmt, None, C.byref(p))
        assert st == -1 and not p.value
    assert L.spmv_exec_f32(None, None, mx.SPMV_OP_NORMAL, 1.0, None, 0.0, None) == -1
    assert L.spmv_exec_f64(None, None, mx.SPMV_OP_TRANSPOSE, 1.0, None, 0.0, None) == -1


def test_reference_partition_count(mx):
    import oracle
    for rows, nnz in ((0, 0), (10, 5), (1000, 31000), (8388608, 185000000), (16777216, 449455096)):
        assert mx.lib().spmv_merge_default_partitions(rows, nnz) == oracle.merge_default_partitions(rows, nnz)


def test_generators_deterministic_across_thread_counts(mx):
    from muxi_spmv_gb300 import workloads as W
    for name in ("poisson16k", "powerlaw8m", "stencil3d_256"):
        s = W.scaled(name, 3000, seed=5)
        a = mx.generate(s, threads=1)
        b = mx.generate(s, threads=5)
        assert all(np.array_equal(p, q) for p, q in zip(a, b))
    x1 = mx.gen_vector(10001, 3, threads=1)
    x2 = mx.gen_vector(10001, 3, threads=4)
    assert np.array_equal(x1, x2) and x1.min() >= -1 and x1.max() <= 1


def test_generator_laws(mx):
    from muxi_spmv_gb300 import workloads as W
    rp, ci, v = mx.generate(W.spec("poisson16k"))
    lens = np.diff(rp)
    assert lens.min() >= 1 and lens.max() <= 64 and abs(lens.mean() - 12.0) < 0.1
    for r in range(0, 16384, 97):
        row = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0)  # sorted, without replacement
    assert np.all(np.abs(v) <= 1.0)
    rp, ci, v = mx.generate(W.scaled("stencil2d_4096", 64 * 64))
    assert len(ci) == 5 * 64 * 64 - 4 * 64
    rp, ci, v = mx.generate(W.scaled("stencil3d_256", 16 ** 3))
    assert len(ci) == (3 * 16 - 2) ** 3
    s = W.scaled("powerlaw8m", 50000, seed=1)
    rp, ci, v = mx.generate(s)
    assert np.all(np.diff(rp) >= 1) and np.all(ci >= 0) and np.all(ci < s.numCols)
    lens = np.diff(rp)
    assert lens.max() <= s.p1
