"""Build the uhm_gb300 native library in-tree (uhm_gb300/libuhm_gb300.so).

All CUDA code targets sm_103a only.  Translation units compile in parallel
into uhm_gb300/_build/, then link into one shared library that exports the C
ABI of include/uhm_gb300.h.  Usage: ``python -m uhm_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libuhm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = [
    "mesh.cpp",
    "sparse.cpp",
    "fill.cpp",
    "capi.cpp",
    "engine.cu",
    "k_factor.cu",
    "k_solve.cu",
    "k_tc_gemm.cu",
    "k_chol_tc.cu",
    "k_noalloc.cu",
    "k_selector.cu",
    "k_elements.cu",
]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _flags(src: str):
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-O3",
              "-I" + SRC, "-I" + os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        return ARCH + common + ["--expt-relaxed-constexpr", "-Xptxas", "-O3"]
    return ["-x", "c++"] + common


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".hpp", ".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "uhm_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(SRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([nvcc, "-c", src, "-o", obj] + _flags(s))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
