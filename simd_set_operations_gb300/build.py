"""Builds libsetops_gpu.so in-tree for sm_103a (GB300).

    python simd_set_operations_gb300/build.py

Translation units are compiled in parallel into ``_build/`` and linked with
the static CUDA runtime into ``simd_set_operations_gb300/libsetops_gpu.so``.
A unit is recompiled only when it or a header is newer than its object.
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
LIB = PKG / "libsetops_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra",
             "-Wno-unused-parameter", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    units = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    tasks = []
    objs = []
    for src in units:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if not _stale(obj, src, headers):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        else:
            cxx = os.environ.get("CXX", "g++")
            cmd = [cxx, *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
        tasks.append(cmd)
    if tasks:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            for cmd, fut in [(c, ex.submit(_run, c)) for c in tasks]:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
                fut.result()
    if tasks or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp),
              *map(str, objs), "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
