"""Build libdgsip.so in-tree for sm_103a with nvcc (no cmake, no torch extension).

    python -m dg_nn_public_gb300.build          # or __graft_entry__.build()

Translation units compile in parallel; the result lands in
dg_nn_public_gb300/_lib/libdgsip.so.  A rebuild happens only when a source
is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libdgsip.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dg_host.cpp", "dg_serve.cpp", "dg_solver.cu"]
HEADERS = ["dg_internal.h", "dg_kernels.cuh", "dg_kernels2.cuh", "dg_mixed.cuh", "dg_batched.cuh", "dg_batched_tc.cuh",
           "dg_noalloc.cuh", "dg_vcycle_cluster.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdgsip")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in _sources()] + \
        [os.path.join(CSRC, h) for h in HEADERS if os.path.exists(os.path.join(CSRC, h))] + \
        [os.path.join(INCLUDE, "dgsip.h"), os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    obj_dir = os.path.join(LIBDIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]

    def compile_one(src):
        out = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + common + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, src), "-o", out]
        if src.endswith(".cpp"):
            cmd = [nvcc] + common + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", out]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        return out

    with cf.ThreadPoolExecutor(max_workers=len(_sources())) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
