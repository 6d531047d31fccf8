"""Builds libswgb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel; the shared library lands next to
this file.  No CMake, no torch extension machinery: the library is a plain
C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
BUILD = HERE / "_build"
LIB = HERE / "libswgb300.so"

SOURCES = ["api.cu", "acoustic.cu", "elastic.cu", "vd.cu", "cpml.cpp", "noalloc.cu", "dense.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or Path(cand).exists()):
            return cand
    return "nvcc"


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (src + ".o")
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "swgb300.h"]
    newest = max(d.stat().st_mtime for d in deps)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
