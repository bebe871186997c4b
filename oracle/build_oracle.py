"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/libsdb_oracle.so``: the C restatement (sdb_oracle.c), built
  with gcc -O3 -fopenmp.  Portable C, so it builds the same on x86-64 and on
  aarch64.
* ``oracle/_ref/libsdb_ref.so``: the reference's own kernel headers
  (kernels/*.hpp and kernels/types.cpp of the SYCLDB repository), compiled
  where they lie against the host SYCL shim in ``oracle/ref_shim``.  Built
  only when the reference checkout is present (``SYCLDB_REFERENCE`` or
  /root/reference); it is a checker for the restatement, never a product path.

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
REFERENCE = os.environ.get("SYCLDB_REFERENCE", "/root/reference")


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


def main():
    print(build_oracle(verbose=True))
    r = build_ref(verbose=True)
    print(r if r else "reference checkout not present: oracle/_ref not built")


if __name__ == "__main__":
    sys.exit(main())
