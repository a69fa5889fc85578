"""Build libforcegpu.so (the C-ABI engine) for sm_103a, in-tree.

    python d3-force-3d-webgpu_gb300/build.py [--verbose-ptxas]

Each .cu file of csrc/ compiles in parallel with nvcc (-gencode arch=compute_103a,code=sm_103a),
then they link into forcegpu/libforcegpu.so, next to the Python bindings that load it. The
objects go to _build/ (git-ignored). Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "forcegpu", "libforcegpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libforcegpu.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "forcegpu.h"))
    return max(os.path.getmtime(h) for h in hs)


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or verbose_ptxas or not os.path.exists(obj) or \
                os.path.getmtime(obj) < max(os.path.getmtime(src), hdr):
            cmd = [cc, "-c", src, "-o", obj] + ARCH + FLAGS
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        failed = [(c, r) for c, r in zip(jobs, results) if r.returncode != 0]
        for c, r in zip(jobs, results):
            if verbose_ptxas or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
        if failed:
            raise RuntimeError("nvcc failed on " + ", ".join(os.path.basename(c[2]) for c, _ in failed))
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call([cc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="--verbose-ptxas" in sys.argv, force="--force" in sys.argv))
