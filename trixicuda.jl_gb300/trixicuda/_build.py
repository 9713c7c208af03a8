"""Builds libtrixi_b200.so (sm_103a) in-tree with nvcc.

Every translation unit under ``csrc/`` is compiled in parallel to
``_build/obj`` and linked into ``_build/libtrixi_b200.so``; an object is
rebuilt when its source or any header is newer.  The measurement
diagnostics under ``csrc/diag/`` (FMA-peak probe, conversion check) are
linked into a separate ``_build/libtrixi_diag.so`` that only the benchmark
and the tests load.  Nothing is installed into site-packages.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # trixicuda.jl_gb300/
CSRC = PKG_ROOT / "csrc"
INCLUDE = PKG_ROOT.parent / "include"
BUILD = PKG_ROOT / "_build"
LIB_NAME = "libtrixi_b200.so"
DIAG_NAME = "libtrixi_diag.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def library_path() -> Path:
    return BUILD / LIB_NAME


def diag_library_path() -> Path:
    return BUILD / DIAG_NAME


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libtrixi_b200.so")
    return cand


def _newest_header() -> float:
    hdrs = (list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) +
            list((CSRC / "diag").glob("*.h")))
    return max((h.stat().st_mtime for h in hdrs), default=0.0)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    obj_dir = BUILD / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hdr_time = _newest_header()
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (("diag_" if src.parent.name == "diag" else "") + src.stem + ".o")
        if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_time):
            return obj
        cmd = [nvcc, *common, *ARCH_FLAGS, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compiling {src.name} failed:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout, res.stderr)
        return obj

    diag_sources = sorted((CSRC / "diag").glob("*.cu"))
    workers = jobs or max(1, min(len(sources) + len(diag_sources), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs_all = list(ex.map(compile_one, sources + diag_sources))
    objs, diag_objs = objs_all[:len(sources)], objs_all[len(sources):]

    def link(path: Path, name: str, parts) -> None:
        if path.exists() and path.stat().st_mtime >= max(o.stat().st_mtime for o in parts):
            return
        tmp = path.with_suffix(".so.tmp")
        cmd = [nvcc, "-shared", *ARCH_FLAGS, "-o", str(tmp), *map(str, parts)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"linking {name} failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, path)

    link(library_path(), LIB_NAME, objs)
    if diag_objs:
        link(diag_library_path(), DIAG_NAME, diag_objs)
    return library_path()


if __name__ == "__main__":
    print(build(verbose=True))
