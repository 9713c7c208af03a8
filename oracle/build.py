"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``trixi_oracle.c`` with gcc + OpenMP into ``oracle/_build/liboracle.so``.
The reference (TrixiCUDA.jl) is pure Julia with its arithmetic in the
un-vendored Trixi.jl, so no reference source can be compiled here; the
oracle is a C restatement (see trixi_oracle.c's header).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"


def build() -> Path:
    src = HERE / "trixi_oracle.c"
    hdr = HERE / "trixi_oracle.h"
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-std=c11", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
