"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/libsdb_oracle.so``: the C restatement (sdb_oracle.c), built
  with gcc -O3 -fopenmp.  Portable C, so it builds the same on x86-64 and on
  aarch64.
* ``oracle/_ref/libsdb_ref.so``: the reference's own kernel headers
  (kernels/*.hpp and kernels/types.cpp of the SYCLDB repository), compiled
  where they lie against the host SYCL shim in ``oracle/ref_shim``.  Built
  only when the reference checkout is present (``SYCLDB_REFERENCE``, else a
  ``reference`` directory beside the repository's own); it is a checker for
  the restatement, never a product path.
* ``oracle/_ref/libsdb_ref_exec.so`` and ``libsdb_ref_exec_seg4096.so``: the
  reference's own executor (executor/, operations/preprocessing.cpp and
  memory_manager.cpp, runtime/runtime.cpp, models/*.hpp through them,
  kernels/types.cpp and jit_kernels.cpp, app/query_utils.cpp,
  gen-cpp/calciteserver_types.cpp) compiled where it lies against the host
  shims of ``oracle/ref_shim`` (SYCL, Thrift types, the disabled JIT), in its
  correctness mode (``ref_exec_prefix.hpp``), with ``ref_exec.cpp`` as the
  client; the second with 4096-row segments.  Also only with the checkout.

Usage: ``python oracle/build_oracle.py`` (idempotent; rebuilds when sources
are newer than the output).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The SYCLDB checkout: SYCLDB_REFERENCE, else <parent of the repository>/reference.
REFERENCE = os.environ.get("SYCLDB_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _newer(out: str, srcs) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def build_oracle(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "sdb_oracle.c")
    out = os.path.join(BUILD, "libsdb_oracle.so")
    if _newer(out, [src]):
        cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", out + ".tmp", src]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(out + ".tmp", out)
    return out


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE, "kernels", "selection.hpp"))


def build_ref(verbose: bool = False):
    """Compile the reference kernels against the host shim.  Returns the
    library path, or None when the reference checkout is absent."""
    if not reference_available():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "libsdb_ref.so")
    srcs = [os.path.join(HERE, "ref_kernels.cpp"), os.path.join(HERE, "ref_shim", "sycl", "sycl.hpp"),
            os.path.join(REFERENCE, "kernels", "types.cpp")]
    srcs += [os.path.join(REFERENCE, "kernels", f) for f in
             ("selection.hpp", "projection.hpp", "aggregation.hpp", "join.hpp", "common.hpp", "types.hpp")]
    if _newer(out, srcs):
        cmd = ["g++", "-O1", "-std=c++20", "-fPIC", "-shared", "-w",
               "-I", os.path.join(HERE, "ref_shim"), "-I", REFERENCE,
               "-o", out + ".tmp",
               os.path.join(HERE, "ref_kernels.cpp"), os.path.join(REFERENCE, "kernels", "types.cpp")]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(out + ".tmp", out)
    return out


EXEC_SOURCES = ("executor/ddor_executor.cpp", "executor/result_writer.cpp", "operations/preprocessing.cpp",
                "operations/memory_manager.cpp", "runtime/runtime.cpp", "kernels/types.cpp", "kernels/jit_kernels.cpp",
                "app/query_utils.cpp", "gen-cpp/calciteserver_types.cpp")


def build_ref_exec(segment_rows: int = 0, verbose: bool = False):
    """Compile the reference's executor against the host shims (its
    translation units in parallel).  segment_rows > 0 replaces its
    SEGMENT_SIZE.  Returns the library path, or None without the checkout."""
    if not reference_available():
        return None
    from concurrent.futures import ThreadPoolExecutor

    tag = "_seg%d" % segment_rows if segment_rows else ""
    objdir = os.path.join(REF_OUT, "exec" + tag)
    os.makedirs(objdir, exist_ok=True)
    out = os.path.join(REF_OUT, "libsdb_ref_exec%s.so" % tag)
    shim = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(HERE, "ref_shim")) for f in fs]
    units = [os.path.join(REFERENCE, u) for u in EXEC_SOURCES] + [os.path.join(HERE, "ref_exec.cpp")]
    headers = [os.path.join(REFERENCE, d, f) for d in ("models", "executor", "operations", "kernels", "runtime")
               for f in os.listdir(os.path.join(REFERENCE, d)) if f.endswith((".hpp", ".h"))]
    deps = shim + headers + [os.path.join(HERE, "ref_exec_prefix.hpp"), os.path.join(REFERENCE, "common.hpp")]
    flags = ["g++", "-std=c++17", "-O1", "-fPIC", "-w", "-include", os.path.join(HERE, "ref_exec_prefix.hpp"),
             "-I", os.path.join(HERE, "ref_shim"), "-I", REFERENCE]
    if segment_rows:
        flags.append("-DREF_EXEC_SEGMENT_SIZE=%d" % segment_rows)

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        if _newer(obj, [src] + deps):
            cmd = flags + ["-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd))
            subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, units))
    if _newer(out, objs):
        subprocess.check_call(["g++", "-shared", "-o", out + ".tmp"] + objs)
        os.replace(out + ".tmp", out)
    return out


def main():
    print(build_oracle(verbose=True))
    r = build_ref(verbose=True)
    print(r if r else "reference checkout not present: oracle/_ref not built")
    for seg in (0, 4096):
        r = build_ref_exec(seg, verbose=True)
        if r:
            print(r)


if __name__ == "__main__":
    sys.exit(main())
