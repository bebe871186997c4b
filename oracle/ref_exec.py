"""The reference's own executor as a checker (TEST INFRASTRUCTURE ONLY).

``oracle/_ref/libsdb_ref_exec.so`` is SYCLDB's executor
(executor/ddor_executor.cpp and everything it calls, built by
``build_oracle.build_ref_exec`` from the reference checkout against the host
shims of ``oracle/ref_shim``).  ``run`` writes a dataset in the reference's
columnar layout (one raw int32 file per column, ``<NAME><i>``), runs a plan
through ``execute_ddor_plan`` with the reference's host placement (primary
device -1) and reads back the ``.res`` rows it saves.  Tests only: nothing in
the product imports this module.
"""
from __future__ import annotations

import ctypes
import json
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def library(segment_rows: int = 0) -> str:
    tag = "_seg%d" % segment_rows if segment_rows else ""
    return os.path.join(HERE, "_ref", "libsdb_ref_exec%s.so" % tag)


def available(segment_rows: int = 0) -> bool:
    return os.path.exists(library(segment_rows))


_LIBS = {}


def _lib(segment_rows: int):
    if segment_rows not in _LIBS:
        L = ctypes.CDLL(library(segment_rows))
        L.ref_exec_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
                                   ctypes.c_size_t]
        L.ref_exec_run.restype = ctypes.c_int
        _LIBS[segment_rows] = L
    return _LIBS[segment_rows]


def write_tables(directory: str, tables) -> None:
    """tables: {name: {column index: int32 array}} -> <NAME><i> files."""
    for name, cols in tables.items():
        for c, a in cols.items():
            np.ascontiguousarray(a, dtype=np.int32).tofile(os.path.join(directory, "%s%d" % (name.upper(), c)))


def run(tables, plan, segment_rows: int = 0, on_device: bool = False):
    """Rows of the reference executor's result for `plan` over `tables`,
    sorted (the canonical order of the other checkers)."""
    L = _lib(segment_rows)
    with tempfile.TemporaryDirectory() as d:
        write_tables(d, tables)
        err = ctypes.create_string_buffer(1024)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            rc = L.ref_exec_run(d.encode(), json.dumps(plan).encode(), b"q", 1 if on_device else 0, err, len(err))
        finally:
            os.chdir(cwd)
        if rc != 0:
            raise RuntimeError("reference executor: " + err.value.decode(errors="replace"))
        with open(os.path.join(d, "q.res")) as f:
            rows = [tuple(int(x) for x in line.split()) for line in f if line.strip()]
    rows.sort()
    return rows
