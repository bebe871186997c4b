"""ctypes bindings of the C ABI declared in ``include/sycldb_gpu.h``.

The native library is the product: every call here goes to
``sycldb_gb300/_build/libsycldb_gb300.so``.  There is no Python or CPU
fallback; if the library is missing, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32, c_uint64, c_void_p

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsycldb_gb300.so")

SDB_OK = 0
SDB_ERR_INVALID = -1
SDB_ERR_CUDA = -2
SDB_ERR_NOMEM = -3
SDB_ERR_TIMEOUT = -4
SDB_ERR_UNSUPPORTED = -5
SDB_ERR_DEVICE = -6

EQ, NE, LT, LE, GT, GE = range(6)
NONE, AND, OR = range(3)
MUL, DIV, ADD, SUB = range(4)

SRC_COL, SRC_REG, SRC_LIT = range(3)
# sdb_op_kernel: the operator-at-a-time kernels whose launch shape is tuned
OP_KERNELS = ("fill_u8", "select_lit", "select_cols", "logical", "fill_i32", "binop", "sum", "count_flags", "min_max",
              "occ_to_flags", "build_keys", "probe_semi", "build_kv", "probe_full", "gather")
OP_SELECT, OP_SEARCH_RANGE, OP_SEARCH_POINTS, OP_SEMI_PROBE, OP_FULL_PROBE, OP_BINOP, OP_FILL = range(7)
TERM_FLAGS, TERM_SUM, TERM_GROUPBY, TERM_BUILD_KEYS, TERM_BUILD_KV = range(5)
CHAIN_MAX_OPS, CHAIN_MAX_REGS, CHAIN_MAX_KEYS = 16, 8, 4


class SdbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("sycldb status %d: %s" % (status, message))
        self.status = status


class Operand(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("reg", c_int32), ("lit", c_int32), ("pad", c_int32), ("col", c_void_p)]


class ChainOp(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("cmp_op", c_int32), ("logic_op", c_int32), ("bin_op", c_int32),
                ("a", Operand), ("b", Operand), ("lo", c_int32), ("hi", c_int32), ("out_reg", c_int32),
                ("ht_log2", c_int32), ("ht", c_void_p), ("out_col", c_void_p)]


class ChainDesc(ctypes.Structure):
    _fields_ = [("n", c_uint64), ("flags_in", c_void_p), ("flags_out", c_void_p), ("n_ops", c_int32),
                ("terminal", c_int32), ("ops", ChainOp * CHAIN_MAX_OPS), ("value", Operand), ("sum_out", c_void_p),
                ("n_keys", c_int32), ("pad", c_int32), ("keys", Operand * CHAIN_MAX_KEYS),
                ("key_min", c_int32 * CHAIN_MAX_KEYS), ("key_max", c_int32 * CHAIN_MAX_KEYS), ("P", c_uint64),
                ("out_keys", c_void_p * CHAIN_MAX_KEYS), ("out_sum", c_void_p), ("occ", c_void_p),
                ("build_key", Operand), ("build_val", Operand), ("ht_out", c_void_p), ("ht_min", c_int32),
                ("ht_len", c_int32), ("ht_zeroed", c_int32), ("ht_log2", c_int32)]


class EngineConfig(ctypes.Structure):
    _fields_ = [("arena_bytes", c_uint64), ("segment_rows", c_uint64), ("fuse", c_int32), ("profile", c_int32),
                ("stream", c_void_p), ("plan_cache", c_int32), ("order_by", c_int32), ("join_tables", c_int32),
                ("no_shared_scans", c_int32)]


class BatchStats(ctypes.Structure):
    _fields_ = [("n_plans", c_int32), ("kernels_per_run", c_int32), ("graph", c_int32), ("chain_launches", c_int32),
                ("batched_chains", c_int32), ("batched_builds", c_int32), ("arena_bytes", c_uint64), ("zero_bytes", c_uint64),
                ("host_bytes", c_uint64), ("last_run_ms", c_double), ("last_chain_ms", c_double),
                ("last_pre_ms", c_double), ("last_post_ms", c_double), ("last_build_ms", c_double),
                ("paired_chains", c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", c_uint64), ("pinned_bytes", c_uint64), ("slots", c_int32), ("max_batch", c_int32),
                ("streams_per_slot", c_int32), ("no_direct", c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [(f, c_uint64) for f in ("submitted", "completed", "failed", "batches", "batched_plans",
                                        "max_batch_plans", "max_inflight_plans", "peak_device_bytes",
                                        "peak_pinned_bytes", "budget_bytes", "direct_plans", "sizing_us",
                                        "launch_us", "paired_chains")]


SDB_BATCH_EAGER = 1
SDB_BATCH_NO_CHAIN_BATCH = 2
SDB_BATCH_BUILDS_ONLY = 4

_P = c_void_p  # device pointers travel as integers
_SIGS = {
    "sdb_last_error": (c_char_p, []),
    "sdb_version": (c_char_p, []),
    "sdb_abi_sizeof": (c_size_t, [c_char_p]),
    "sdb_launch_count": (c_uint64, []),
    "sdb_device_errors": (c_int, [POINTER(c_uint64), _P]),
    "sdb_fill_u8": (c_int, [_P, c_uint64, c_uint8, _P]),
    "sdb_select_lit": (c_int, [_P, c_int32, c_int, c_int, _P, _P, c_uint64, _P]),
    "sdb_select_cols": (c_int, [_P, _P, c_int, c_int, _P, _P, c_uint64, _P]),
    "sdb_logical": (c_int, [c_int, _P, _P, _P, c_uint64, _P]),
    "sdb_fill_i32": (c_int, [_P, c_int32, c_uint64, _P]),
    "sdb_binop_cc": (c_int, [_P, _P, _P, c_int, _P, c_uint64, _P]),
    "sdb_binop_lc": (c_int, [_P, c_int32, _P, c_int, _P, c_uint64, _P]),
    "sdb_binop_cl": (c_int, [_P, _P, c_int32, c_int, _P, c_uint64, _P]),
    "sdb_sum_i32_u64": (c_int, [_P, _P, c_uint64, _P, _P]),
    "sdb_groupby_sum": (c_int, [POINTER(c_void_p), POINTER(c_int32), POINTER(c_int32), c_int, _P, _P, c_uint64,
                                c_uint64, POINTER(c_void_p), _P, _P, _P]),
    "sdb_occ_to_flags": (c_int, [_P, _P, c_uint64, _P]),
    "sdb_ht_build_keys": (c_int, [_P, _P, c_uint64, _P, c_int32, c_int32, _P]),
    "sdb_probe_semi": (c_int, [_P, _P, _P, c_uint64, _P, c_int32, c_int32, _P]),
    "sdb_ht_build_kv": (c_int, [_P, _P, _P, c_uint64, _P, c_int32, c_int32, _P]),
    "sdb_probe_full": (c_int, [_P, _P, _P, _P, c_uint64, _P, c_int32, c_int32, _P]),
    "sdb_oa_log2_slots": (c_int, [c_uint64]),
    "sdb_ht_build_keys_oa": (c_int, [_P, _P, c_uint64, _P, c_int, c_int32, c_int32, c_int, _P]),
    "sdb_probe_semi_oa": (c_int, [_P, _P, _P, c_uint64, _P, c_int, c_int32, c_int32, _P]),
    "sdb_ht_build_kv_oa": (c_int, [_P, _P, _P, c_uint64, _P, c_int, c_int32, c_int32, c_int, _P]),
    "sdb_probe_full_oa": (c_int, [_P, _P, _P, _P, c_uint64, _P, c_int, c_int32, c_int32, _P]),
    "sdb_compact_scratch_bytes": (c_size_t, [c_uint64]),
    "sdb_compact_row_ids": (c_int, [_P, c_uint64, _P, _P, _P, c_size_t, _P]),
    "sdb_compact_row_ids_noalloc": (c_int, [_P, c_uint64, _P, _P, _P]),
    "sdb_gather_i32": (c_int, [_P, _P, _P, _P, c_uint64, _P]),
    "sdb_gather_u64": (c_int, [_P, _P, _P, _P, c_uint64, _P]),
    "sdb_count_flags": (c_int, [_P, c_uint64, _P, _P]),
    "sdb_min_max_i32": (c_int, [_P, c_uint64, _P, _P]),
    "sdb_compact_gather": (c_int, [_P, c_uint64, c_int, POINTER(c_void_p), POINTER(c_int), POINTER(c_void_p), _P,
                                   _P]),
    "sdb_compact_gather_occ": (c_int, [_P, c_uint64, c_int, POINTER(c_void_p), POINTER(c_int), POINTER(c_void_p), _P,
                                       _P]),
    "sdb_sort_scratch_bytes": (c_size_t, [c_uint64]),
    "sdb_sort_rows": (c_int, [POINTER(c_void_p), POINTER(c_int), POINTER(c_int), c_int, c_uint64, _P, _P, c_size_t,
                              _P]),
    "sdb_fused_chain": (c_int, [POINTER(ChainDesc), _P]),
    "sdb_fused_chain_variant": (c_int, [POINTER(ChainDesc), c_int, _P]),
    "sdb_chain_tune_set": (c_int, [c_int, c_int, c_uint64, c_int]),
    "sdb_chain_tune_get": (c_int, [c_int, c_int, c_uint64]),
    "sdb_chain_tune_set_op": (c_int, [c_int, c_int, c_int, c_uint64, c_int]),
    "sdb_chain_tune_get_op": (c_int, [c_int, c_int, c_int, c_uint64]),
    "sdb_chain_registers": (c_int, [POINTER(ChainDesc)]),
    "sdb_chain_specialised": (c_int, [POINTER(ChainDesc)]),
    "sdb_chain_pairable": (c_int, [POINTER(ChainDesc), POINTER(ChainDesc)]),
    "sdb_chain_pair_key": (c_int, [POINTER(ChainDesc), POINTER(c_uint64)]),
    "sdb_chain_launch_pair": (c_int, [POINTER(ChainDesc), POINTER(ChainDesc), c_void_p]),
    "sdb_fused_launch_counts": (c_int, [POINTER(c_uint64), POINTER(c_uint64)]),
    "sdb_chain_batch_scratch_bytes": (c_size_t, [POINTER(ChainDesc), c_int]),
    "sdb_chain_batch_create": (c_int, [POINTER(ChainDesc), c_int, _P, c_size_t, _P, POINTER(c_void_p)]),
    "sdb_chain_batch_create_async": (c_int, [POINTER(ChainDesc), c_int, _P, c_size_t, c_void_p, c_size_t, _P,
                                             POINTER(c_void_p)]),
    "sdb_chain_batch_launch": (c_int, [c_void_p, _P]),
    "sdb_chain_batch_launch_part": (c_int, [c_void_p, c_int, _P]),
    "sdb_chain_batch_kernels": (c_int, [c_void_p]),
    "sdb_chain_batch_destroy": (None, [c_void_p]),
    "sdb_gen_uniform_host": (c_int32, [c_uint64, c_uint64, c_uint64, c_int32, c_int32]),
    "sdb_gen_uniform": (c_int, [_P, c_uint64, c_uint64, c_uint64, c_uint64, c_int32, c_int32, _P]),
    "sdb_gen_uniform_cpu": (c_int, [_P, c_uint64, c_uint64, c_uint64, c_uint64, c_int32, c_int32]),
    "sdb_gen_datekeys_cpu": (c_int, [_P, c_uint64, c_int64]),
    "sdb_gen_dates": (c_int, [_P, c_uint64, c_uint64, c_uint64, c_uint64, c_int32, _P]),
    "sdb_gen_dates_cpu": (c_int, [_P, c_uint64, c_uint64, c_uint64, c_uint64, c_int32]),
    "sdb_plan_check": (c_int, [c_char_p, POINTER(c_int), POINTER(c_int), c_int]),
    "sdb_op_tune_set": (c_int, [c_int, c_uint64, c_int, c_int]),
    "sdb_op_tune_get": (c_int, [c_int, c_uint64, POINTER(c_int), POINTER(c_int)]),
    "sdb_plan_to_idl_json": (c_int, [c_char_p, c_char_p, c_size_t, POINTER(c_size_t)]),
    "sdb_engine_create": (c_int, [POINTER(EngineConfig), POINTER(c_void_p)]),
    "sdb_engine_destroy": (c_int, [c_void_p]),
    "sdb_engine_load_table": (c_int, [c_void_p, c_char_p, c_int, POINTER(c_void_p), c_uint64, c_int]),
    "sdb_engine_execute": (c_int, [c_void_p, c_char_p, POINTER(c_void_p)]),
    "sdb_engine_load_dir": (c_int, [c_void_p, c_char_p, c_char_p, c_uint64, c_int]),
    "sdb_engine_sync_tables": (c_int, [c_void_p]),
    "sdb_result_shape": (c_int, [c_void_p, POINTER(c_int), POINTER(c_uint64)]),
    "sdb_result_column": (c_int, [c_void_p, c_int, POINTER(c_int), POINTER(c_void_p)]),
    "sdb_result_write_res": (c_int, [c_void_p, c_char_p]),
    "sdb_result_free": (None, [c_void_p]),
    "sdb_engine_kernel_stats": (c_int, [c_void_p, c_int, POINTER(c_char_p), POINTER(c_uint64), POINTER(c_double)]),
    "sdb_engine_last_plan_ms": (c_int, [c_void_p, POINTER(c_double)]),
    "sdb_engine_batch_prepare": (c_int, [c_void_p, POINTER(c_char_p), c_int, c_int, POINTER(c_void_p)]),
    "sdb_batch_run": (c_int, [c_void_p, POINTER(c_void_p)]),
    "sdb_batch_info": (c_int, [c_void_p, POINTER(BatchStats)]),
    "sdb_batch_free": (None, [c_void_p]),
    "sdb_batch_layout": (c_int, [c_void_p, c_int, POINTER(c_int), POINTER(c_int), c_int, POINTER(c_int)]),
    "sdb_batch_segment": (c_int, [c_void_p, c_int, c_int, POINTER(c_uint64), POINTER(c_uint64), c_int,
                                  POINTER(c_uint64)]),
    "sdb_batch_host": (c_void_p, [c_void_p, POINTER(c_size_t)]),
    "sdb_server_create": (c_int, [c_void_p, POINTER(ServerConfig), POINTER(c_void_p)]),
    "sdb_server_submit": (c_int, [c_void_p, c_char_p, POINTER(c_int64)]),
    "sdb_server_next": (c_int, [c_void_p, c_int, POINTER(c_int64), POINTER(c_int), POINTER(c_void_p),
                                POINTER(c_double)]),
    "sdb_server_stats_get": (c_int, [c_void_p, POINTER(ServerStats)]),
    "sdb_server_destroy": (c_int, [c_void_p]),
    "sdb_server_replay": (c_int, [c_void_p, POINTER(c_char_p), POINTER(c_double), c_int, POINTER(c_int),
                                  POINTER(c_void_p), POINTER(c_double), POINTER(c_double)]),
    "sdb_engine_replay_plain": (c_int, [c_void_p, POINTER(c_char_p), POINTER(c_double), c_int, POINTER(c_int),
                                        POINTER(c_void_p), POINTER(c_double), POINTER(c_double)]),
}

_LIB = None


def lib():
    """Loads the native library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("sycldb_gb300 native library not built: %s "
                               "(run `python -m sycldb_gb300.build`)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        for cls, name in ((Operand, "sdb_operand"), (ChainOp, "sdb_chain_op"), (ChainDesc, "sdb_chain_desc"),
                          (EngineConfig, "sdb_engine_config"), (BatchStats, "sdb_batch_stats"),
                          (ServerConfig, "sdb_server_config"), (ServerStats, "sdb_server_stats")):
            n = L.sdb_abi_sizeof(name.encode())
            if n != ctypes.sizeof(cls):
                raise RuntimeError("ABI mismatch for %s: C %d, ctypes %d" % (name, n, ctypes.sizeof(cls)))
        _LIB = L
    return _LIB


def exported_symbols():
    return sorted(_SIGS)


def last_error() -> str:
    return lib().sdb_last_error().decode()


def check(status: int):
    if status != SDB_OK:
        raise SdbError(status, last_error())
    return status


def fused_launch_counts() -> tuple:
    """(launches of the shape-specialised passes, of those the bound passes)
    since the library loaded."""
    a, b = c_uint64(0), c_uint64(0)
    check(lib().sdb_fused_launch_counts(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def force_chain_variant(variant: int):
    """Sets every tuning-table entry to `variant`.  -1 restores the process's
    table: the built-in defaults, then the committed autotuner table again if
    an engine of this process loaded it."""
    L = lib()
    for term in range(3):
        for nregs in (1, 4, 8):
            for b in range(40):
                check(L.sdb_chain_tune_set(term, nregs, 1 << b, variant))
    if variant == -1:
        from . import engine

        if engine._TUNING_LOADED:
            from . import autotune

            autotune.load_default()


def plan_to_idl(plan) -> dict:
    """A plan in either dialect the executor reads (IDL shape or Calcite
    RelJson), as the executor parsed it, in the IDL shape."""
    import json

    text = (plan if isinstance(plan, str) else json.dumps(plan)).encode()
    L = lib()
    n = c_size_t(0)
    check(L.sdb_plan_to_idl_json(text, None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    check(L.sdb_plan_to_idl_json(text, buf, n.value + 1, ctypes.byref(n)))
    return json.loads(buf.value.decode())
