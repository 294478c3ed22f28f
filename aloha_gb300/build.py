"""Builds libaloha_gb300.so (the C ABI + sm_103a kernels) in-tree with nvcc.

Every translation unit is compiled in parallel into ``aloha_gb300/_build``
and linked into ``aloha_gb300/libaloha_gb300.so``.  Device code is built with
``-fmad=false`` (every fused multiply-add is written out as fmaf) and host code
with ``-ffp-contract=off``, so results are bit-identical on every machine.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libaloha_gb300.so")
SOURCES = ["render.cu", "schedule.cu", "api.cpp", "order.cpp", "batch.cpp", "adjoint.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build aloha_gb300")


def _flags(src: str, verbose_ptxas: bool) -> list[str]:
    f = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-fmad=false",
         "-I", CSRC, "-I", os.path.join(PKG, "..", "include")]
    if src.endswith(".cu"):
        f += ARCH + ["-lineinfo"]
        if verbose_ptxas:
            f += ["-Xptxas", "-v"]
    return f


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(PKG, "..", "include", "aloha.h"))
    return os.path.getmtime(obj) < max(os.path.getmtime(d) for d in deps if os.path.exists(d))


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []
    todo = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or verbose_ptxas or _stale(obj, src):
            todo.append([cc, "-c", src, "-o", obj] + _flags(s, verbose_ptxas))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, max(1, len(todo)))) as ex:
        for cmd, r in ex.map(run, todo):
            logs.append(r.stderr)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if todo or not os.path.exists(LIB):
        link = [cc, "-shared", "-o", LIB] + objs + ARCH + ["-Xlinker", "--no-undefined", "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    if verbose_ptxas:
        sys.stderr.write("".join(logs))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
