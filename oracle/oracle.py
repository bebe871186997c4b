"""CPU oracle for the SYCLDB operator path (TEST INFRASTRUCTURE ONLY).

This module is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference legs of ``bench.py`` import it; the product
(``sycldb_gb300``) never does.

It has two layers:

* ``lib()`` loads ``oracle/_build/libsdb_oracle.so`` (``sdb_oracle.c``), the
  per-row restatement of every reference kernel, and wraps each one over numpy
  buffers.
* ``OracleExecutor`` restates the reference executor: plan-node dispatch
  (executor/ddor_executor.cpp:22-245), execution info and DAG order
  (operations/preprocessing.cpp:14-275) and the TransientTable operators
  (models/transient_table.hpp:750-1927), with the column statistics of
  models/models.hpp.  Kernels run as soon as they are enqueued: on one device
  the reference's deferred per-segment phases (transient_table.hpp:347-506)
  read and write the same buffers in the same order, so deferral does not
  change any result.

Parity status: the kernel restatements are pinned against the reference's own
kernel functors, compiled here from kernels/*.hpp against a host SYCL shim
(``oracle/_ref``, see ``build_oracle.py``).  The executor layer cannot be
compiled here (it needs AdaptiveCpp, oneDPL and Thrift); it is checked by an
independent naive evaluator in the tests, not by the reference itself.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsdb_oracle.so")

SEGMENT_SIZE = 1 << 28  # common.hpp:12

# kernels/selection.hpp:7-21, kernels/aggregation.hpp:11-17
EQ, NE, LT, LE, GT, GE = range(6)
NONE, AND, OR = range(3)
MUL, DIV, ADD, SUB = range(4)

# kernels/types.cpp:3-21
TABLE_COLUMN_INDICES = {
    "lineorder": {2, 3, 4, 5, 8, 9, 11, 12, 13},
    "part": {0, 2, 3, 4},
    "supplier": {0, 3, 4, 5},
    "customer": {0, 3, 4, 5},
    "ddate": {0, 4, 5},
}
TABLE_COLUMN_NUMBERS = {"lineorder": 17, "part": 9, "supplier": 7, "customer": 8, "ddate": 17}


def base_name(name: str) -> str:
    """Tables may be named "<schema table>@<tag>"; the schema is the part before '@'."""
    return name.split("@", 1)[0]


def get_comp_op(op: str) -> int:
    """kernels/selection.hpp:23-39 (unknown operators map to EQ)."""
    return {"==": EQ, ">=": GE, "<=": LE, "<": LT, ">": GT, "!=": NE, "<>": NE}.get(op, EQ)


def get_logical_op(op: str) -> int:
    """kernels/selection.hpp:41-49 (anything else is NONE)."""
    return {"AND": AND, "OR": OR}.get(op, NONE)


def is_filter_logical(op: str) -> bool:
    """kernels/selection.hpp:53-59: all-alphabetic operator names are logical."""
    return all(c.isalpha() for c in op)


def get_op_from_string(op: str) -> int:
    """kernels/aggregation.hpp:37-48."""
    table = {"*": MUL, "/": DIV, "+": ADD, "-": SUB}
    if op not in table:
        raise ValueError("Unknown operation: " + op)
    return table[op]


def stoi(s: str) -> int:
    """std::stoi: optional whitespace and sign, then leading decimal digits."""
    t = s.strip()
    i = 0
    if i < len(t) and t[i] in "+-":
        i += 1
    j = i
    while j < len(t) and t[j].isdigit():
        j += 1
    if j == i:
        raise ValueError("stoi: no conversion: %r" % s)
    v = int(t[:j])
    if not -(2 ** 31) <= v < 2 ** 31:
        raise OverflowError("stoi: out of range: %r" % s)
    return v


def to_i32(v: int) -> int:
    """C conversion of an int64 literal to int (modular)."""
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= (1 << 31) else v


# --------------------------------------------------------------------------
# C kernel library
# --------------------------------------------------------------------------
_LIB = None

_P_I32 = ctypes.POINTER(ctypes.c_int32)
_P_U8 = ctypes.POINTER(ctypes.c_uint8)
_P_U32 = ctypes.POINTER(ctypes.c_uint32)
_P_U64 = ctypes.POINTER(ctypes.c_uint64)
_PP_I32 = ctypes.POINTER(_P_I32)


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle library missing: %s (run oracle/build_oracle.py)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        u64, i32, i = ctypes.c_uint64, ctypes.c_int32, ctypes.c_int
        sig = {
            "o_fill_u8": (None, [_P_U8, u64, ctypes.c_uint8]),
            "o_select_lit": (None, [_P_I32, i32, i, i, _P_U8, _P_U8, u64]),
            "o_select_cols": (None, [_P_I32, _P_I32, i, i, _P_U8, _P_U8, u64]),
            "o_logical_kernel": (None, [i, _P_U8, _P_U8, _P_U8, u64]),
            "o_fill_i32": (None, [_P_I32, i32, u64]),
            "o_binop_cc": (None, [_P_I32, _P_I32, _P_I32, i, _P_U8, u64]),
            "o_binop_lc": (None, [_P_I32, i32, _P_I32, i, _P_U8, u64]),
            "o_binop_cl": (None, [_P_I32, _P_I32, i32, i, _P_U8, u64]),
            "o_sum_i32_u64": (None, [_P_I32, _P_U8, u64, _P_U64]),
            "o_groupby_sum": (ctypes.c_int64, [_PP_I32, _P_I32, _P_I32, i, _P_I32, _P_U8, u64, u64,
                                               _PP_I32, _P_U64, _P_U32]),
            "o_occ_to_flags": (None, [_P_U32, _P_U8, u64]),
            "o_ht_build_keys": (ctypes.c_int64, [_P_I32, _P_U8, u64, _P_U8, i32, i32]),
            "o_probe_semi": (None, [_P_I32, _P_U8, _P_U8, u64, _P_U8, i32, i32]),
            "o_ht_build_kv": (ctypes.c_int64, [_P_I32, _P_I32, _P_U8, u64, _P_I32, i32, i32]),
            "o_probe_full": (None, [_P_I32, _P_I32, _P_U8, _P_U8, u64, _P_I32, i32, i32]),
            "o_compact_row_ids": (None, [_P_U8, u64, _P_I32, _P_U32]),
            "o_gather_i32": (None, [_P_I32, _P_I32, ctypes.c_uint32, _P_I32]),
            "o_count_flags": (ctypes.c_uint64, [_P_U8, u64]),
            "o_min_max": (None, [_P_I32, u64, _P_I32, _P_I32]),
            "o_num_threads": (ctypes.c_int, []),
            "o_gen_uniform": (None, [_P_I32, u64, u64, u64, u64, i32, i32]),
            "o_gen_dates": (None, [_P_I32, u64, u64, u64, u64, i32]),
            "o_gen_datekeys": (None, [_P_I32, u64, ctypes.c_int64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


class OracleGen:
    """The seeded column generator restated in sdb_oracle.c, with the
    interface of ``sycldb_gb300.ssb.LibGen``: the CPU legs of the benchmark
    generate their inputs with it and load nothing of the native library."""

    @staticmethod
    def _dst(a: np.ndarray, n: int):
        assert a.dtype == np.int32 and a.size >= n and a.flags["C_CONTIGUOUS"]
        return _p(a, ctypes.c_int32)

    def uniform(self, a, n, row0, seed, sid, lo, hi):
        if hi < lo:
            raise ValueError("uniform: hi < lo")
        lib().o_gen_uniform(self._dst(a, n), n, row0, seed, sid, lo, hi)

    def dates(self, a, n, row0, seed, sid, ndays):
        if ndays < 1:
            raise ValueError("dates: ndays < 1")
        lib().o_gen_dates(self._dst(a, n), n, row0, seed, sid, ndays)

    def datekeys(self, a, n, day0):
        lib().o_gen_datekeys(self._dst(a, n), n, day0)


def _p(a: np.ndarray, ctype):
    assert a.flags["C_CONTIGUOUS"], "oracle buffers must be contiguous"
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def p_i32(a):
    assert a.dtype == np.int32
    return _p(a, ctypes.c_int32)


def p_u8(a):
    assert a.dtype == np.uint8
    return _p(a, ctypes.c_uint8)


def p_u32(a):
    assert a.dtype == np.uint32
    return _p(a, ctypes.c_uint32)


def p_u64(a):
    assert a.dtype == np.uint64
    return _p(a, ctypes.c_uint64)


# Thin numpy-level wrappers (also used directly by the kernel parity tests).
def select_lit(col, v, cmp, logic, fin, fout):
    lib().o_select_lit(p_i32(col), to_i32(v), cmp, logic, p_u8(fin), p_u8(fout), col.size)


def select_cols(a, b, cmp, logic, fin, fout):
    lib().o_select_cols(p_i32(a), p_i32(b), cmp, logic, p_u8(fin), p_u8(fout), a.size)


def logical(logic, fin, local, fout):
    lib().o_logical_kernel(logic, p_u8(fin), p_u8(local), p_u8(fout), fin.size)


def fill_i32(dst, v):
    lib().o_fill_i32(p_i32(dst), to_i32(v), dst.size)


def binop_cc(res, a, b, op, flags):
    lib().o_binop_cc(p_i32(res), p_i32(a), p_i32(b), op, p_u8(flags), res.size)


def binop_lc(res, lit, b, op, flags):
    lib().o_binop_lc(p_i32(res), to_i32(lit), p_i32(b), op, p_u8(flags), res.size)


def binop_cl(res, a, lit, op, flags):
    lib().o_binop_cl(p_i32(res), p_i32(a), to_i32(lit), op, p_u8(flags), res.size)


def sum_i32_u64(col, flags, acc: np.ndarray):
    lib().o_sum_i32_u64(p_i32(col), p_u8(flags), col.size, p_u64(acc))


def groupby_sum(keys, mins, maxs, val, flags, P, out_keys, out_sum, occ):
    g = len(keys)
    kp = (_P_I32 * g)(*[p_i32(k) for k in keys])
    okp = (_P_I32 * g)(*[p_i32(k) for k in out_keys])
    mn = np.ascontiguousarray(mins, dtype=np.int32)
    mx = np.ascontiguousarray(maxs, dtype=np.int32)
    return lib().o_groupby_sum(kp, p_i32(mn), p_i32(mx), g, p_i32(val), p_u8(flags), val.size,
                               P, okp, p_u64(out_sum), p_u32(occ))


def occ_to_flags(occ, flags):
    lib().o_occ_to_flags(p_u32(occ), p_u8(flags), occ.size)


def ht_build_keys(key, flags, ht, mn, length):
    return lib().o_ht_build_keys(p_i32(key), p_u8(flags), key.size, p_u8(ht), mn, length)


def probe_semi(key, fin, fout, ht, mn, mx):
    lib().o_probe_semi(p_i32(key), p_u8(fin), p_u8(fout), key.size, p_u8(ht), mn, mx)


def ht_build_kv(key, val, flags, ht2, mn, length):
    return lib().o_ht_build_kv(p_i32(key), p_i32(val), p_u8(flags), key.size, p_i32(ht2), mn, length)


def probe_full(key, val_out, fin, fout, ht2, mn, mx):
    lib().o_probe_full(p_i32(key), p_i32(val_out), p_u8(fin), p_u8(fout), key.size, p_i32(ht2), mn, mx)


def compact_row_ids(flags):
    ids = np.empty(flags.size, dtype=np.int32)
    cnt = ctypes.c_uint32(0)
    lib().o_compact_row_ids(p_u8(flags), flags.size, p_i32(ids), ctypes.byref(cnt))
    return ids[: cnt.value]


def count_flags(flags):
    return int(lib().o_count_flags(p_u8(flags), flags.size))


def min_max(col):
    mn, mx = ctypes.c_int32(0), ctypes.c_int32(0)
    lib().o_min_max(p_i32(col), col.size, ctypes.byref(mn), ctypes.byref(mx))
    return mn.value, mx.value


# --------------------------------------------------------------------------
# Storage model (models/models.hpp)
# --------------------------------------------------------------------------
@dataclass
class OSegment:
    """Segment: models/models.hpp:20-1069.  ``data`` is int32, or uint64 for
    aggregate results."""
    data: Optional[np.ndarray]
    min: int = 0
    max: int = 0
    is_aggregate_result: bool = False

    @property
    def nrows(self):
        return 0 if self.data is None else self.data.size


@dataclass
class OColumn:
    """Column: models/models.hpp:1072-1649."""
    segments: List[OSegment] = field(default_factory=list)
    is_aggregate_result: bool = False

    def get_min_max(self):
        """models/models.hpp:1257-1272."""
        if self.is_aggregate_result:
            raise RuntimeError("can't get min/max of aggregate result column")
        return (min(s.min for s in self.segments), max(s.max for s in self.segments))

    def full(self) -> np.ndarray:
        return np.concatenate([s.data for s in self.segments]) if self.segments else np.empty(0, np.int32)


def _split(n: int, seg: int):
    """Segment layout of Column ctors: models/models.hpp:1083-1096."""
    out, start = [], 0
    while start < n:
        out.append((start, min(seg, n - start)))
        start += seg
    return out


def column_from_data(data: np.ndarray, seg: int) -> OColumn:
    """Base column with per-segment min/max computed at load (models/models.hpp:38-78)."""
    col = OColumn()
    for start, cnt in _split(data.size, seg):
        d = data[start:start + cnt]
        mn, mx = min_max(d)
        col.segments.append(OSegment(d, mn, mx))
    return col


def materialized_column(n: int, seg: int) -> OColumn:
    """Materialized column (models/models.hpp:1098-1122).  The reference leaves
    the contents uninitialised; the oracle zero-fills them."""
    col = OColumn()
    for _start, cnt in _split(n, seg):
        col.segments.append(OSegment(np.zeros(cnt, dtype=np.int32)))
    return col


@dataclass
class OTable:
    """Table: models/models.hpp:1652-1802.  Columns not supplied stay empty."""
    name: str
    columns: List[OColumn]
    nrows: int


def make_table(name: str, cols: Dict[int, np.ndarray], seg: int = SEGMENT_SIZE) -> OTable:
    ncols = TABLE_COLUMN_NUMBERS[base_name(name)]
    nrows = None
    columns = []
    for i in range(ncols):
        if i in cols:
            d = np.ascontiguousarray(cols[i], dtype=np.int32)
            if nrows is None:
                nrows = d.size
            if d.size != nrows:
                raise ValueError("column length mismatch in %s%d" % (name, i))
            columns.append(column_from_data(d, seg))
        else:
            columns.append(OColumn())
    return OTable(name, columns, nrows or 0)


# --------------------------------------------------------------------------
# Execution info (operations/preprocessing.cpp)
# --------------------------------------------------------------------------
def parse_expression_columns(expr, columns: set):
    """operations/preprocessing.cpp:5-12."""
    if expr["exprType"] == "COLUMN":
        columns.add(int(expr["input"]))
    elif expr["exprType"] == "EXPR":
        for o in expr.get("operands", []):
            parse_expression_columns(o, columns)


def dag_topological_sort(rels) -> List[int]:
    """operations/preprocessing.cpp:14-102.  The lineorder scan is pushed back
    while other nodes remain."""
    n = len(rels)
    dag = [[0] * n for _ in range(n)]
    S: List[int] = []  # deque: index 0 = front
    for rel in rels:
        op = rel["relOp"]
        rid = int(rel["id"])
        if op == "TABLE_SCAN":
            S.insert(0, rid)
        elif op in ("FILTER", "PROJECT", "AGGREGATE", "SORT"):
            dag[rid - 1][rid] = 1
        elif op == "JOIN":
            if len(rel["inputs"]) != 2:
                return []
            dag[int(rel["inputs"][0])][rid] = 1
            dag[int(rel["inputs"][1])][rid] = 1
        else:
            return []
    order = []
    while S:
        node = S.pop()
        if S and rels[node]["relOp"] == "TABLE_SCAN" and base_name(rels[node]["tables"][1]) == "lineorder":
            S.insert(0, node)
            continue
        order.append(node)
        for i in range(n):
            if dag[node][i] == 1:
                dag[node][i] = 0
                if not any(dag[j][i] == 1 for j in range(n)):
                    S.insert(0, i)
    if len(order) != n:
        return []
    return order


def parse_execution_info(rels):
    """operations/preprocessing.cpp:104-275 (the parts that drive execution:
    loaded columns, group-by column per table, DAG order)."""
    loaded: Dict[str, set] = {}
    group_by: Dict[str, int] = {}
    ops_info: List[List[tuple]] = []
    for rel in rels:
        op = rel["relOp"]
        if op == "TABLE_SCAN":
            t = rel["tables"][1]
            ops_info.append([(t, i) for i in range(TABLE_COLUMN_NUMBERS[base_name(t)])])
            loaded[t] = set()
        elif op == "FILTER":
            info = list(ops_info[-1])
            cols: set = set()
            parse_expression_columns(rel["condition"], cols)
            for c in cols:
                loaded[info[c][0]].add(info[c][1])
            ops_info.append(info)
        elif op == "PROJECT":
            last = ops_info[-1]
            info = []
            for e in rel["exprs"]:
                cols = set()
                parse_expression_columns(e, cols)
                for c in cols:
                    loaded[last[c][0]].add(last[c][1])
                if cols:
                    info.append(last[min(cols)])
            ops_info.append(info)
        elif op == "AGGREGATE":
            last = ops_info[-1]
            info = []
            for g in rel["group"]:
                t, ci = last[g]
                loaded[t].add(ci)
                info.append((t, ci))
                group_by[t] = ci
            for agg in rel["aggs"]:
                for c in agg["operands"]:
                    loaded[last[c][0]].add(last[c][1])
                info.append(last[agg["operands"][0]])
            ops_info.append(info)
        elif op == "JOIN":
            left = ops_info[int(rel["inputs"][0])]
            right = ops_info[int(rel["inputs"][1])]
            cols = set()
            parse_expression_columns(rel["condition"], cols)
            for c in cols:
                t, ci = left[c] if c < len(left) else right[c - len(left)]
                loaded[t].add(ci)
            ops_info.append(list(left) + list(right))
        elif op == "SORT":
            info = list(ops_info[-1])
            for col in rel.get("collation", []):
                f = int(col["field"])
                if f < len(info):
                    loaded[info[f][0]].add(info[f][1])
            ops_info.append(info)
        else:
            ops_info.append([])
    return loaded, group_by, dag_topological_sort(rels)


# --------------------------------------------------------------------------
# TransientTable (models/transient_table.hpp)
# --------------------------------------------------------------------------
class OTransientTable:
    def __init__(self, base: OTable, seg: int):
        # ctor: models/transient_table.hpp:52-156 (flags filled with true)
        self.seg = seg
        self.nrows = base.nrows
        self.flags = np.ones(self.nrows, dtype=np.uint8)
        self.current_columns: List[Optional[OColumn]] = list(base.columns)
        self.group_by_column: Optional[OColumn] = None
        self.group_by_column_index = 0

    def segs(self):
        return _split(self.nrows, self.seg)

    def set_group_by_column(self, col: int):
        """models/transient_table.hpp:190-194."""
        self.group_by_column = self.current_columns[col]
        self.group_by_column_index = col

    # Each flag-producing phase writes the secondary buffer and swaps it in
    # (transient_table.hpp:300-326); here a fresh output array plays that role.
    def apply_filter(self, expr, parent_op: str):
        """models/transient_table.hpp:750-981."""
        if expr["exprType"] != "EXPR":
            return
        op = expr["op"]
        if op == "SEARCH":
            col = self.current_columns[int(expr["operands"][0]["input"])]
            rs = expr["operands"][1]["literal"]["rangeSet"]
            out = np.empty_like(self.flags)
            logic = get_logical_op(parent_op)
            for si, (start, cnt) in enumerate(self.segs()):
                data = col.segments[si].data
                local = np.empty(cnt, dtype=np.uint8)
                # Segment::search_operator: models/models.hpp:604-718
                if len(rs) == 1:
                    lo, hi = stoi(rs[0][1]), stoi(rs[0][2])
                    select_lit(data, lo, GE, NONE, local, local)
                    select_lit(data, hi, LE, AND, local, local)
                else:
                    a, b = stoi(rs[0][1]), stoi(rs[1][1])
                    select_lit(data, a, EQ, NONE, local, local)
                    select_lit(data, b, EQ, OR, local, local)
                fin = self.flags[start:start + cnt]
                fo = out[start:start + cnt]
                logical(logic, fin, local, fo)
            self.flags = out
        elif is_filter_logical(op):
            used = False
            for operand in expr["operands"]:
                self.apply_filter(operand, op if used else parent_op)
                used = True
        else:
            ops = expr["operands"]
            if len(ops) != 2:
                return
            cols: List[Optional[OColumn]] = [None, None]
            literal = False
            lit = 0
            for i in range(2):
                t = ops[i]["exprType"]
                if t == "COLUMN":
                    cols[i] = self.current_columns[int(ops[i]["input"])]
                elif t == "LITERAL":
                    literal = True
                    lit = to_i32(int(ops[i]["literal"]["value"]))
                else:
                    return
            if cols[0] is None:
                raise ValueError("filter comparison needs a column as its first operand")
            cmp, logic = get_comp_op(op), get_logical_op(parent_op)
            out = np.empty_like(self.flags)
            for si, (start, cnt) in enumerate(self.segs()):
                fin = self.flags[start:start + cnt]
                fo = out[start:start + cnt]
                if literal:
                    select_lit(cols[0].segments[si].data, lit, cmp, logic, fin, fo)
                else:
                    select_cols(cols[0].segments[si].data, cols[1].segments[si].data, cmp, logic, fin, fo)
            self.flags = out

    def apply_project(self, exprs):
        """models/transient_table.hpp:983-1224."""
        new_columns: List[Optional[OColumn]] = []
        for i, expr in enumerate(exprs):
            t = expr["exprType"]
            if t == "COLUMN":
                new_columns.append(self.current_columns[int(expr["input"])])
                if int(expr["input"]) == self.group_by_column_index:
                    self.group_by_column_index = i
            elif t == "LITERAL":
                v = to_i32(int(expr["literal"]["value"]))
                col = materialized_column(self.nrows, self.seg)
                for s in col.segments:  # Segment::fill_with_literal: models/models.hpp:293-326
                    fill_i32(s.data, v)
                    s.min = s.max = v
                new_columns.append(col)
            elif t == "EXPR":
                ops = expr["operands"]
                if len(ops) != 2:
                    return
                bop = get_op_from_string(expr["op"])
                col = materialized_column(self.nrows, self.seg)
                k0, k1 = ops[0]["exprType"], ops[1]["exprType"]
                for si, (start, cnt) in enumerate(self.segs()):
                    res = col.segments[si]
                    fl = self.flags[start:start + cnt]
                    # Segment::perform_operator: models/models.hpp:760-845
                    if k0 == "COLUMN" and k1 == "COLUMN":
                        a = self.current_columns[int(ops[0]["input"])].segments[si]
                        b = self.current_columns[int(ops[1]["input"])].segments[si]
                        res.min, res.max = min(a.min, b.min), max(a.max, b.max)
                        binop_cc(res.data, a.data, b.data, bop, fl)
                    elif k0 == "LITERAL" and k1 == "COLUMN":
                        b = self.current_columns[int(ops[1]["input"])].segments[si]
                        res.min, res.max = b.min, b.max
                        binop_lc(res.data, to_i32(int(ops[0]["literal"]["value"])), b.data, bop, fl)
                    elif k0 == "COLUMN" and k1 == "LITERAL":
                        a = self.current_columns[int(ops[0]["input"])].segments[si]
                        res.min, res.max = a.min, a.max
                        binop_cl(res.data, a.data, to_i32(int(ops[1]["literal"]["value"])), bop, fl)
                    else:
                        return
                new_columns.append(col)
        self.current_columns = new_columns

    def apply_aggregate(self, agg, group):
        """models/transient_table.hpp:1226-1647."""
        acol = self.current_columns[int(agg["operands"][0])]
        if len(group) == 0:
            acc = np.zeros(1, dtype=np.uint64)
            for si, (start, cnt) in enumerate(self.segs()):
                sum_i32_u64(acol.segments[si].data, self.flags[start:start + cnt], acc)
            self.nrows = 1
            self.flags = np.ones(1, dtype=np.uint8)
            self.current_columns = [OColumn([OSegment(acc, is_aggregate_result=True)], True)]
            return
        gcols = [self.current_columns[int(g)] for g in group]
        mins, maxs = [], []
        P = 1
        for c in gcols:
            mn, mx = c.get_min_max()
            mins.append(mn)
            maxs.append(mx)
            P *= (to_i32(mx - mn + 1)) & 0xFFFFFFFFFFFFFFFF
            P &= 0xFFFFFFFFFFFFFFFF
        if P > (1 << 31):
            raise MemoryError("group-by slot array too large: %d" % P)
        out_sum = np.zeros(P, dtype=np.uint64)
        occ = np.zeros(P, dtype=np.uint32)
        out_keys = [np.zeros(P, dtype=np.int32) for _ in gcols]
        for si, (start, cnt) in enumerate(self.segs()):
            groupby_sum([c.segments[si].data for c in gcols], mins, maxs, acol.segments[si].data,
                        self.flags[start:start + cnt], P, out_keys, out_sum, occ)
        flags = np.empty(P, dtype=np.uint8)
        occ_to_flags(occ, flags)
        self.nrows = P
        self.flags = flags
        new_cols: List[Optional[OColumn]] = []
        for k in out_keys:
            c = OColumn()
            for start, cnt in _split(P, self.seg):
                c.segments.append(OSegment(k[start:start + cnt], 0, 0))
            new_cols.append(c)
        ac = OColumn(is_aggregate_result=True)
        for start, cnt in _split(P, self.seg):
            ac.segments.append(OSegment(out_sum[start:start + cnt], is_aggregate_result=True))
        new_cols.append(ac)
        self.current_columns = new_cols

    def apply_join(self, right: "OTransientTable", rel):
        """models/transient_table.hpp:1649-1927."""
        cond = rel["condition"]
        left_column = int(cond["operands"][0]["input"])
        right_column = int(cond["operands"][1]["input"]) - len(self.current_columns)
        if not (0 <= left_column < len(self.current_columns)
                and 0 <= right_column < len(right.current_columns)):
            raise ValueError("Invalid column indices in join condition.")
        probe = self.current_columns[left_column]
        build = right.current_columns[right_column]
        mn, mx = build.get_min_max()
        length = to_i32(mx - mn + 1)
        if rel.get("joinType", "") == "semi":
            # Column::build_keys_hash_table: models/models.hpp:1413-1452
            ht = np.zeros(max(length, 0), dtype=np.uint8)
            for si, (start, cnt) in enumerate(right.segs()):
                ht_build_keys(build.segments[si].data, right.flags[start:start + cnt], ht, mn, length)
            out = np.empty_like(self.flags)
            # Column::semi_join: models/models.hpp:1454-1507
            for si, (start, cnt) in enumerate(self.segs()):
                probe_semi(probe.segments[si].data, self.flags[start:start + cnt],
                           out[start:start + cnt], ht, mn, mx)
            self.flags = out
            self.current_columns.extend([None] * len(right.current_columns))
        else:
            gb = right.group_by_column
            if gb is None:
                raise ValueError("inner join needs a group-by column on the build side")
            gmin, gmax = gb.get_min_max()
            new_col = materialized_column(self.nrows, self.seg)
            gidx = len(self.current_columns) + right.group_by_column_index
            self.current_columns.extend([None] * len(right.current_columns))
            self.current_columns[gidx] = new_col
            # Column::build_key_vals_hash_table: models/models.hpp:1509-1548
            ht2 = np.zeros(2 * max(length, 0), dtype=np.int32)
            for si, (start, cnt) in enumerate(right.segs()):
                ht_build_kv(build.segments[si].data, gb.segments[si].data,
                            right.flags[start:start + cnt], ht2, mn, length)
            out = np.empty_like(self.flags)
            # Column::full_join_operation: models/models.hpp:1550-1648
            for si, (start, cnt) in enumerate(self.segs()):
                seg = new_col.segments[si]
                probe_full(probe.segments[si].data, seg.data, self.flags[start:start + cnt],
                           out[start:start + cnt], ht2, mn, mx)
                seg.min, seg.max = gmin, gmax
            self.flags = out

    def result_rows(self):
        """Rows as the result writer emits them: flagged rows in row order, the
        non-null columns in order (executor/result_writer.cpp:41-67).
        Returns a list of numpy arrays (one per output column)."""
        sel = np.nonzero(self.flags)[0]
        out = []
        for c in self.current_columns:
            if c is None:
                continue
            full = np.concatenate([s.data for s in c.segments]) if c.segments else None
            if full is None:
                raise RuntimeError("result column has no data")
            out.append(full[sel])
        return out


class OracleExecutor:
    """execute_ddor_plan restated: executor/ddor_executor.cpp:22-245."""

    def __init__(self, tables: Dict[str, OTable], segment_size: int = SEGMENT_SIZE):
        self.tables = tables
        self.seg = segment_size

    def execute(self, plan) -> List[np.ndarray]:
        if isinstance(plan, str):
            plan = json.loads(plan)
        rels = plan["rels"]
        _loaded, group_by, order = parse_execution_info(rels)
        if not order:
            raise ValueError("DAG topological sort failed")
        output_table = [-1] * len(rels)
        tts: List[OTransientTable] = []
        for rel in rels:
            if rel["relOp"] != "TABLE_SCAN":
                continue
            name = rel["tables"][1]
            base = self.tables[name]
            tt = OTransientTable(base, self.seg)
            if name in group_by:
                tt.set_group_by_column(group_by[name])
            tts.append(tt)
            output_table[int(rel["id"])] = len(tts) - 1
        for rid in order:
            rel = rels[rid]
            op = rel["relOp"]
            if op == "TABLE_SCAN":
                continue
            if op == "FILTER":
                t = output_table[rid - 1]
                tts[t].apply_filter(rel["condition"], "")
                output_table[rid] = t
            elif op == "PROJECT":
                t = output_table[rid - 1]
                tts[t].apply_project(rel["exprs"])
                output_table[rid] = t
            elif op == "AGGREGATE":
                t = output_table[rid - 1]
                tts[t].apply_aggregate(rel["aggs"][0], rel["group"])
                output_table[rid] = t
            elif op == "JOIN":
                lt = output_table[int(rel["inputs"][0])]
                rt = output_table[int(rel["inputs"][1])]
                tts[lt].apply_join(tts[rt], rel)
                output_table[rid] = lt
            elif op == "SORT":
                output_table[rid] = output_table[rid - 1]
        return tts[output_table[len(rels) - 1]].result_rows()


def canonical_rows(cols: Sequence[np.ndarray]):
    """Rows as tuples of Python ints, sorted: the canonical form compared by
    the parity tests."""
    if not cols:
        return []
    rows = list(zip(*[c.tolist() for c in cols]))
    rows.sort()
    return rows
