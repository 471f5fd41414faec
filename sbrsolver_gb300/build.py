"""Builds ``sbrsolver_gb300/libsbr.so`` in-tree: the CUDA engine and C ABI
(include/sbr.h), compiled for sm_103a only.

Host code is compiled with -ffp-contract=off: the scene preparation must
round every FP64 product and sum separately, like the reference.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libsbr.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def newer(target: str, sources) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_library(force: bool = False, verbose: bool = False) -> str:
    srcs = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))]
    srcs.append(os.path.join(ROOT, "include", "sbr.h"))
    if not force and newer(LIB, srcs):
        return LIB
    nvcc = _nvcc()
    obj_dir = os.path.join(PKG, "_build")
    os.makedirs(obj_dir, exist_ok=True)
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math"]
    jobs = [
        [nvcc, *ARCH, *common, "-lineinfo", "-c", os.path.join(CSRC, "sbr_engine.cu"),
         "-o", os.path.join(obj_dir, "sbr_engine.o")],
        [nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, "sbr_host.cpp"),
         "-o", os.path.join(obj_dir, "sbr_host.o")],
        [nvcc, *ARCH, *common, "-lineinfo", "-c", os.path.join(CSRC, "sbr_noalloc.cu"),
         "-o", os.path.join(obj_dir, "sbr_noalloc.o")],
        [nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, "sbr_server.cpp"),
         "-o", os.path.join(obj_dir, "sbr_server.o")],
        [nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, "sbr_io.cpp"),
         "-o", os.path.join(obj_dir, "sbr_io.o")],
        [nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, "sbr_pattern.cpp"),
         "-o", os.path.join(obj_dir, "sbr_pattern.o")],
    ]
    with ThreadPoolExecutor(len(jobs)) as ex:
        outs = list(ex.map(run, jobs))
    if verbose:
        print("".join(outs))
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, os.path.join(obj_dir, "sbr_engine.o"),
         os.path.join(obj_dir, "sbr_host.o"), os.path.join(obj_dir, "sbr_noalloc.o"),
         os.path.join(obj_dir, "sbr_server.o"), os.path.join(obj_dir, "sbr_io.o"),
         os.path.join(obj_dir, "sbr_pattern.o")])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print("built", build_library(force="-f" in sys.argv, verbose="-v" in sys.argv))
