"""The C++ drop-in layer: tests/cpp/test_dropin.cu uses the reference's call
sites (namespace muxi_spmv, CSRMatrix<T>, spmv_csr<T>, csr5_preprocess<T>,
spmv_merge_based<T>, csr_to_ellpack<T>, spmv_exec<T>, reorderColumns ...)
unchanged against include/muxi_spmv.hpp.  Compiling is checked on any
machine; running needs the GPU."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "test_dropin.cu"


def nvcc():
    from muxi_spmv_gb300 import build
    return str(build.cuda_home() / "bin" / "nvcc")


def compile_dropin(out: Path, link: bool):
    from muxi_spmv_gb300 import build
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-I", str(ROOT / "include"),
           str(SRC), "-o", str(out)]
    if link:
        lib = build.build()
        cmd += ["-L", str(lib.parent), "-lmuxispmv", "-Xlinker", f"-rpath={lib.parent}"]
    else:
        cmd.insert(1, "-c")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_dropin_compiles(tmp_path):
    compile_dropin(tmp_path / "dropin.o", link=False)


@pytest.mark.gpu
def test_dropin_runs(tmp_path, mx, cuda):
    exe = compile_dropin(tmp_path / "dropin", link=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAILED" not in r.stdout and r.stdout.strip().endswith("PASSED")
