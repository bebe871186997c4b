"""ctypes access to the reference's own kernel functors (oracle/_ref), built
from kernels/*.hpp of the SYCLDB sources against the host SYCL shim.  Only
available where the reference checkout exists (the CPU container)."""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libsdb_ref.so")

_L = None
P = ctypes.c_void_p


def available() -> bool:
    return os.path.exists(REF_LIB)


def lib():
    global _L
    if _L is None:
        L = ctypes.CDLL(REF_LIB)
        u64, i32, i = ctypes.c_uint64, ctypes.c_int32, ctypes.c_int
        sig = {
            "ref_select_lit": (None, [P, i32, i, i, P, P, u64]),
            "ref_select_lit_str": (None, [P, i32, ctypes.c_char_p, ctypes.c_char_p, P, P, u64]),
            "ref_select_cols": (None, [P, P, i, i, P, P, u64]),
            "ref_logical": (None, [i, P, P, P, u64]),
            "ref_fill_i32": (None, [P, i32, u64]),
            "ref_binop_cc": (None, [P, P, P, i, P, u64]),
            "ref_binop_lc": (None, [P, i32, P, i, P, u64]),
            "ref_binop_cl": (None, [P, P, i32, i, P, u64]),
            "ref_sum_i32_u64": (None, [P, P, u64, P]),
            "ref_groupby_sum": (None, [ctypes.POINTER(P), P, P, i, P, P, u64, u64, ctypes.POINTER(P), P, P]),
            "ref_ht_build_keys": (None, [P, P, u64, P, i32, i32]),
            "ref_probe_semi": (None, [P, P, P, u64, P, i32, i32]),
            "ref_ht_build_kv": (None, [P, P, P, u64, P, i32, i32]),
            "ref_probe_full": (None, [P, P, P, P, u64, P, i32, i32]),
            "ref_count_flags": (ctypes.c_uint64, [P, u64]),
            "ref_get_comp_op": (i, [ctypes.c_char_p]),
            "ref_get_logical_op": (i, [ctypes.c_char_p]),
            "ref_is_filter_logical": (i, [ctypes.c_char_p]),
            "ref_get_binop": (i, [ctypes.c_char_p]),
            "ref_table_column_number": (i, [ctypes.c_char_p]),
            "ref_table_column_loaded": (i, [ctypes.c_char_p, i]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


def ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def ptr_array(arrs):
    return (P * len(arrs))(*[ptr(a) for a in arrs])
