"""Build the in-tree CUDA library librg300.so for sm_103a (nvcc, no CMake).

The three translation units are compiled in parallel and linked into
rismo2d_gb300/librg300.so next to this file.  Re-running is cheap: sources are
only recompiled when they are newer than their object file.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librg300.so")
SOURCES = ["rg_assemble.cu", "rg_linalg.cu", "rg_trsv.cu", "rg_api.cu", "rg_noalloc.cu", "rg_mlp.cu",
           "rg_model.cpp", "rg_wave_layout.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src), os.path.join(CSRC, "rg_internal.cuh"),
            os.path.join(HERE, "..", "include", "rg300.h"), os.path.join(HERE, "..", "include", "rg300_sim.h"),
            os.path.join(HERE, "..", "include", "rg300_mlp.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    if src.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-I/usr/local/cuda/include", "-c"]
    else:
        cmd = [_nvcc()] + ARCH + FLAGS + ["-c"]
    subprocess.check_call(cmd + [os.path.join(CSRC, src), "-o", obj])
    return obj


def build(force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        subprocess.check_call([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
