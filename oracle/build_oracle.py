"""Builds the CPU oracle (oracle.c) into oracle/_build/liboracle.so.

Test infrastructure: the library never links it.  gcc, -O2, -ffp-contract=off
so the FP32 baseline loop and the compensated sums do exactly the operations
written (no fused multiply-add contraction on either x86-64 or AArch64).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"


def build() -> Path:
    OUT.mkdir(exist_ok=True)
    src = HERE / "oracle.c"
    hdr = HERE / "oracle.h"
    if LIB.exists() and LIB.stat().st_mtime > max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    cc = os.environ.get("CC", "gcc")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-o", str(tmp), str(src),
           "-lm", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
