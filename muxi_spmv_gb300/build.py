"""Builds libmuxispmv.so in-tree for sm_103a.

Every CUDA translation unit under csrc/ is compiled by nvcc with one
`-gencode arch=compute_103a,code=sm_103a`; host C++ units by g++.  Units are
compiled in parallel and skipped when their object is newer than every source
and header, so a rebuild after a one-file change takes seconds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libmuxispmv.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _compile(src: Path, obj: Path, cuda: Path, extra: list[str]) -> tuple[Path, str]:
    inc = ["-I", str(INCLUDE), "-I", str(CSRC), "-I", str(cuda / "include")]
    if src.suffix == ".cu":
        # Public symbols are the extern "C" entry points marked visible below.
        cmd = [str(cuda / "bin" / "nvcc"), *ARCH, *NVCC_FLAGS, *extra, *inc, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, ptxas_info: bool = False, jobs: int | None = None) -> Path:
    cuda = cuda_home()
    BUILD.mkdir(exist_ok=True)
    newest = max((h.stat().st_mtime for h in _headers()), default=0.0)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    todo = []
    objs = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if ptxas_info or _stale(obj, src, newest):
            todo.append((src, obj))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, cuda, extra) for s, o in todo]
            for f in futs:
                obj, log = f.result()
                if verbose and log.strip():
                    print(f"--- {obj.name}\n{log}", file=sys.stderr)
    if todo or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
               "-Xlinker", "--no-undefined", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(verbose=True, ptxas_info="--ptxas-info" in sys.argv)
    print(p)
