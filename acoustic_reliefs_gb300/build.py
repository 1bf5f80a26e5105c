"""Builds ``acoustic_reliefs_gb300/lib/libac3d.so`` for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into one shared library with the
static CUDA runtime. Host code is compiled without floating-point contraction so that the tree
and block partition are bit-identical on x86 and Arm hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(OUT_DIR, "libac3d.so")
OBJ_DIR = os.path.join(HERE, "_build")

SOURCES = ["api.cpp", "tree.cpp", "geometry.cu", "assemble.cu", "aca_df.cu", "matvec.cu", "pack.cu", "krylov.cu", "gmres.cu", "listener.cu",
           "adjoint.cu", "noalloc.cu", "serve.cpp", "multi.cu", "tcselftest.cu", "obj.cpp", "texmap.cu", "relief.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _flags(src: str) -> list[str]:
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", "-diag-suppress", "1444",
         "-I", os.path.join(HERE, "..", "include")] + ARCH
    if src.endswith(".cpp"):
        f = ["-x", "cu"] + f
    return f


def _compile(src: str) -> str:
    obj = os.path.join(OBJ_DIR, src + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "ac3d.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + _flags(src) + ["-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(o) for o in objs):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), "-shared", "-Xcompiler", "-fPIC"] + ARCH + objs + ["-o", tmp, "-lcudart_static", "-lrt",
                                                                         "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
