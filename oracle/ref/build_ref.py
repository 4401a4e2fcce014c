"""Recipe: build the reference's own hot-path functions into
oracle/_ref/libmuxi_ref.so, from the sources where they lie under the
reference tree: $MUXI_REF_ROOT, else a `reference` folder beside this
repository's folder.  Without either the recipe is skipped.

This is how the CPU oracle is pinned: tests/test_oracle_pins.py runs both on
the same seeded inputs, and tests/golden/make_golden.py stores the
reference's outputs as fixtures.  Nothing built here is shipped or used by
the library.  Outputs go only to oracle/_ref/.

Parts:
  * ref_tests_colreorder.cu / ref_tests_rowreorder.cu include the reference's
    tests/test_column_reordering.cu and tests/test_row_reordering.cu in place
    (their main() renamed) and call the reorder functions they define;
  * ref_src_host.cu includes src/preprocessing/column_reorder.cuh and
    src/spmv/ellpack/spmv_ellpack.cu in place; ref_host_cudart.cpp gives the
    ELL conversion host-memory cudaMalloc/cudaMemcpy;
  * the reference's CPU CSR loop, written inline in
    tests/deep_analysis_runner.cpp:184-190 (FloatType sum += values*x), is
    read out of that file the same way and wrapped in a function;
  * the merge-path and CSR5 index code (csr5_binary_search_row in
    src/spmv/csr5/spmv_csr5.cuh, csr5_compute_tile_boundaries_kernel,
    merge_path_search and compute_merge_partitions_kernel in
    src/spmv/csr5/spmv_csr5.cu) are device functions in a file that also
    launches kernels, so g++ cannot take the file as a whole.  The recipe
    reads those four definitions out of the reference files at build time,
    writes them into oracle/_ref/gen/ref_index.cpp with host shims for
    __device__/__global__ and the thread indices, and runs each kernel body
    over its grid on the CPU.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libmuxi_ref.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def ref_root() -> Path:
    env = os.environ.get("MUXI_REF_ROOT")
    return Path(env) if env else ORACLE.parent.parent / "reference"  # beside the repository's folder


def available() -> bool:
    r = ref_root()
    return (r / "src" / "spmv" / "csr5" / "spmv_csr5.cu").exists()


def _extract(text: str, signature_regex: str) -> str:
    """Returns the full definition (optional template line + body) whose
    header matches signature_regex, by brace matching."""
    m = re.search(signature_regex, text, re.S)
    if not m:
        raise RuntimeError(f"definition not found: {signature_regex}")
    start = m.start()
    # include a preceding `template<...>` line if present
    prev = text.rfind("\n", 0, start - 1)
    line = text[prev + 1:start].strip()
    if line.startswith("template"):
        start = prev + 1
    i = text.index("{", m.end() - 1)
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[start:j + 1]
    raise RuntimeError("unbalanced braces")


def _extract_block(text: str, head_regex: str) -> str:
    """Returns the statement starting at head_regex through its closing brace."""
    m = re.search(head_regex, text)
    if not m:
        raise RuntimeError(f"block not found: {head_regex}")
    i = text.index("{", m.start())
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():j + 1]
    raise RuntimeError("unbalanced braces")


SHIM = r"""// Generated by oracle/ref/build_ref.py from the reference sources; not committed.
#include <algorithm>
#define __device__
#define __forceinline__ inline
#define __global__
using std::min;
using std::max;
struct RefEmuDim { int x = 0, y = 0, z = 0; };
static thread_local RefEmuDim blockIdx, blockDim, threadIdx;
"""

DRIVERS = r"""
extern "C" void ref_csr5_tiles(const int* rowPtr, int numRows, int nnz, int sigma, int* tile_row_ptr,
                               int* tile_nnz_offset, int numTiles) {
    const int bs = 256;
    blockDim.x = bs;
    for (int b = 0; b * bs < numTiles; ++b)
        for (int t = 0; t < bs; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            csr5_compute_tile_boundaries_kernel<256>(rowPtr, numRows, nnz, sigma, tile_row_ptr, tile_nnz_offset,
                                                     numTiles);
        }
}

extern "C" void ref_merge_partitions(int numRows, int nnz, int numPartitions, int* pos) {
    const int bs = 256;
    blockDim.x = bs;
    const int grid = (numPartitions + 2 + 255) / 256;
    for (int b = 0; b < grid; ++b)
        for (int t = 0; t < bs; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            compute_merge_partitions_kernel(numRows, nnz, numRows + nnz, numPartitions, pos);
        }
}

extern "C" void ref_cpu_spmv_f32(int numRows, const int* rp, const int* ci, const float* v, const float* x,
                                 float* y) {
    ref_cpu_loop<float>(numRows, rp, ci, v, x, y);
}

extern "C" void ref_cpu_spmv_f64(int numRows, const int* rp, const int* ci, const double* v, const double* x,
                                 double* y) {
    ref_cpu_loop<double>(numRows, rp, ci, v, x, y);
}

extern "C" void ref_merge_search(const int* rowPtr, int numRows, int nnz, const int* diag, int count, int* rowIdx,
                                 int* nnzIdx) {
    for (int i = 0; i < count; ++i) merge_path_search(rowPtr, numRows, nnz, diag[i], rowIdx[i], nnzIdx[i]);
}
"""


def _gen_index_tu(root: Path) -> Path:
    cuh = (root / "src/spmv/csr5/spmv_csr5.cuh").read_text()
    cu = (root / "src/spmv/csr5/spmv_csr5.cu").read_text()
    parts = [
        _extract(cuh, r"__device__\s+__forceinline__\s+int\s+csr5_binary_search_row\s*\("),
        _extract(cu, r"__global__\s+void\s+csr5_compute_tile_boundaries_kernel\s*\("),
        _extract(cu, r"__device__\s+__forceinline__\s+void\s+merge_path_search\s*\("),
        _extract(cu, r"__global__\s+void\s+compute_merge_partitions_kernel\s*\("),
    ]
    runner = (root / "tests/deep_analysis_runner.cpp").read_text()
    loop = _extract_block(runner, r"for \(int row = 0; row < matrix\.numRows; row\+\+\) \{")
    parts.append("template <typename FloatType>\n"
                 "void ref_cpu_loop(int numRows, const int* h_rowPtr, const int* h_colIdx, const FloatType* h_values,\n"
                 "                  const FloatType* h_x, FloatType* h_reference) {\n"
                 "    struct { int numRows; } matrix = {numRows};\n    " + loop + "\n}")
    GEN.mkdir(parents=True, exist_ok=True)
    p = GEN / "ref_index.cpp"
    p.write_text(SHIM + "\n\n".join(parts) + "\n" + DRIVERS)
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False) -> Path:
    root = ref_root()
    if not available():
        raise FileNotFoundError(f"reference sources not found under {root}")
    srcs = [HERE / n for n in ("ref_tests_colreorder.cu", "ref_tests_rowreorder.cu", "ref_src_host.cu",
                               "ref_host_cudart.cpp", "build_ref.py")]
    if LIB.exists() and not force and LIB.stat().st_mtime > max(s.stat().st_mtime for s in srcs):
        return LIB
    OUT.mkdir(exist_ok=True)
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    nvcc = str(cuda / "bin" / "nvcc")
    inc = ["-I", str(root / "src"), "-I", str(root)]
    objs = []
    for name in ("ref_tests_colreorder.cu", "ref_tests_rowreorder.cu", "ref_src_host.cu"):
        o = OUT / (name + ".o")
        _run([nvcc, *ARCH, "-O2", "-std=c++14", "-w", "-Xcompiler", "-fPIC", *inc, "-c", str(HERE / name),
              "-o", str(o)])
        objs.append(o)
    o = OUT / "ref_host_cudart.o"
    _run(["g++", "-O2", "-fPIC", "-I", str(cuda / "include"), "-c", str(HERE / "ref_host_cudart.cpp"), "-o", str(o)])
    objs.append(o)
    idx = _gen_index_tu(root)
    o = OUT / "ref_index.o"
    _run(["g++", "-O2", "-fPIC", "-w", "-ffp-contract=off", "-c", str(idx), "-o", str(o)])
    objs.append(o)
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs), "-Xlinker", "-Bsymbolic",
          "-Xlinker", f"-rpath={cuda / 'lib64'}"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
