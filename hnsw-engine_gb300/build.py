"""Build libhnswgpu.so in-tree: sm_103a CUDA kernels + the C++20 host library.

    python hnsw-engine_gb300/build.py        # incremental
    python hnsw-engine_gb300/build.py --force

CUDA sources are compiled with ``nvcc -gencode arch=compute_103a,code=sm_103a``
(one target, no PTX fallback), host sources with g++ -std=c++20.  Every
translation unit is compiled in parallel; the output is
hnsw-engine_gb300/lib/libhnswgpu.so, which exports the C ABIs of
include/hnswgpu.h and include/hnswgpu_device.h and the hnsw:: C++ API.
"""
from __future__ import annotations

import argparse
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "lib" / "obj"
LIB = PKG / "lib" / "libhnswgpu.so"
INCLUDE = REPO / "include"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc") if (CUDA_HOME / "bin" / "nvcc").exists() else "nvcc"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CU_FLAGS = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "--fmad=false", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O3", "-std=c++20", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra", f"-I{INCLUDE}",
             f"-I{CUDA_HOME / 'include'}", "-pthread"]


def sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    return cu, cpp


def headers():
    return list(CSRC.glob("*.cuh")) + list((CSRC / "host").glob("*.hpp")) + list(INCLUDE.rglob("*.h*"))


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, force: bool) -> Path:
    obj = OBJ / (src.name + ".o")
    if not force and not _newer(obj, [src, *headers()]):
        return obj
    if src.suffix == ".cu":
        cmd = [NVCC, *CU_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        flags = list(CXX_FLAGS)
        if src.name == "distance.cpp" and platform.machine() in ("x86_64", "AMD64"):
            # the builder's kernels use fmaf(); give the x86 compiler the FMA unit
            flags += ["-mfma", "-mavx2"]
        cmd = ["g++", *flags, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"compile failed: {src.name}")
    return obj


def build(force: bool = False, jobs: int | None = None) -> Path:
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhnswgpu")
    OBJ.mkdir(parents=True, exist_ok=True)
    cu, cpp = sources()
    srcs = cu + cpp
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or _newer(LIB, objs):
        cmd = [NVCC, GENCODE, "-shared", "-Xcompiler", "-fPIC", "-o", str(LIB), *map(str, objs), "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    print(build(a.force, a.j))
