"""Build libgainls.so in-tree for sm_103a (nvcc, translation units compiled in parallel).

    python gain-mpi_gb300/build.py          # builds gain-mpi_gb300/lib/libgainls.so
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build", platform.machine())
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgainls.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cpp", "threej.cpp", "states.cpp", "fp64_kernels.cu", "split.cu", "noalloc.cu", "adjoint.cu", "linetext.cu", "trove.cpp"]
HEADERS = ["gain_internal.h", "split.h", "linefmt.h", "linemath.cuh"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    deps = [path, os.path.join(ROOT, "include", "gain_ls.h"), os.path.join(ROOT, "include", "gain_trove.h")]
    deps += [os.path.join(CSRC, h) for h in HEADERS]
    deps.append(os.path.abspath(__file__))   # the flags below
    if not _stale(obj, deps):
        return obj
    # host code: no floating-point contraction (the host's line arithmetic rounds every
    # product as the reference's does; aarch64 compilers fuse multiply-adds by default)
    cmd = [nvcc(), "-c", "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include")] + ARCH
    cmd += [path, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    stamp = LIB + ".arch"
    same_arch = os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()
    if not same_arch or _stale(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB + ".tmp"] + ARCH + objs + ["-lcudart_static", "-ldl", "-lpthread", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
        with open(stamp, "w") as f:
            f.write(platform.machine())
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
