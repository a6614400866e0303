"""Build libamdg_gb300.so in-tree for sm_103a.

    python adaptive-multiresolution-dg_gb300/build.py

Compiles the CUDA and host C++ translation units in parallel (one -gencode,
no cmake) and links them into lib/libamdg_gb300.so next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libamdg_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def compile_one(src: str) -> str:
    obj = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "amdg.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    common = ["-std=c++17", "-O3", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + common + ["-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "-Xptxas", "-v", "-c", path, "-o", obj]
    else:
        cmd = ["g++"] + common + ["-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-c", path, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if src.endswith(".cu"):
        with open(obj + ".ptxas.txt", "w") as f:
            f.write(res.stderr)
    return obj


def build_examples() -> list[str]:
    """C++ drivers written against host/amdg_dg.hpp, linked to the library."""
    ex_dir = os.path.join(PKG, "examples")
    outs = []
    for src in sorted(f for f in os.listdir(ex_dir) if f.endswith(".cpp")):
        exe = os.path.join(LIB_DIR, src[:-4])
        cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "host"),
               os.path.join(ex_dir, src), "-o", exe, "-L", LIB_DIR, "-lamdg_gb300", f"-Wl,-rpath,{LIB_DIR}"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"example build failed: {' '.join(cmd)}\n{res.stderr}")
        outs.append(exe)
    return outs


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", LIB] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    build_examples()
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
