"""In-tree build of libpolymlp_gb300.so (nvcc, sm_103a) and of the oracle.

`build()` compiles every CUDA translation unit and the host C++ in parallel
with nvcc (-gencode arch=compute_103a,code=sm_103a) into
pypolymlp_gb300/lib/libpolymlp_gb300.so.  Objects go to pypolymlp_gb300/_build/.
Host code is compiled with -ffp-contract=off so that the translation vectors
and wrapped positions are bit-identical to the reference's.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libpolymlp_gb300.so")

CU_SOURCES = ["xrows.cu", "capi.cu", "gram.cu", "gram_tc.cu", "solve.cu", "eval.cu"]
CPP_SOURCES = ["host/model_tables.cpp", "host/params.cpp", "host/cell.cpp", "host/flat_tables.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = []
    for root, _, files in os.walk(CSRC):
        headers += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "polymlp_gb300.h"))
    inc = ["-I" + CSRC, "-I" + os.path.join(REPO, "include")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "--expt-relaxed-constexpr", *inc, "-c", path, "-o", obj])
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", *inc, "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o, file=sys.stderr)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
