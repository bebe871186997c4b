"""In-tree build of the native library ``sycldb_gb300/_build/libsycldb_gb300.so``.

Device code is compiled for sm_103a only (``-gencode arch=compute_103a,
code=sm_103a``); host code is plain C++17.  Translation units compile in
parallel; the link uses nvcc (static CUDA runtime).  No cmake.

Usage: ``python -m sycldb_gb300.build`` or ``sycldb_gb300.build.build()``.
Set ``SDB_PTXAS_VERBOSE=1`` to print ptxas register/shared-memory usage.
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
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libsycldb_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kernels.cu", "fused.cu", "sort.cu"]
CPP_SOURCES = ["errors.cpp", os.path.join("engine", "engine.cpp"), os.path.join("engine", "server.cpp")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(ROOT, "include", "sycldb_gpu.h")]
    for dp, _dn, fns in os.walk(CSRC):
        hs += [os.path.join(dp, f) for f in fns if f.endswith((".cuh", ".hpp", ".h"))]
    return hs


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    headers = _headers()
    ptxas_v = ["-Xptxas", "-v"] if os.environ.get("SDB_PTXAS_VERBOSE") else []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *ptxas_v, *inc,
               "-c", s, "-o", o]
        jobs.append((s, o, cmd))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "c++", *inc, "-c", s, "-o", o]
        jobs.append((s, o, cmd))

    todo = [j for j in jobs if force or _stale(j[1], j[0], headers)]

    def run(job):
        _s, _o, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        if ptxas_v and r.stderr:
            print(r.stderr, file=sys.stderr)
        return r

    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(todo))) as ex:
            list(ex.map(run, todo))
    objs = [j[1] for j in jobs]
    if force or todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs, "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
