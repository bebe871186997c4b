"""The C-ABI library without a GPU: it loads, exports every entry point that
include/sycldb_gpu.h declares, its struct layouts match the bindings, its host
paths (generator, plan ingestion, argument checks) behave."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from sycldb_gb300 import capi, plans, ssb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "sycldb_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sdb_\w+)\s*\(", text)))


def test_header_declares_the_kernel_entries():
    names = declared_functions()
    for k in ["sdb_fill_u8", "sdb_select_lit", "sdb_select_cols", "sdb_logical", "sdb_fill_i32", "sdb_binop_cc",
              "sdb_binop_lc", "sdb_binop_cl", "sdb_sum_i32_u64", "sdb_groupby_sum", "sdb_occ_to_flags",
              "sdb_ht_build_keys", "sdb_probe_semi", "sdb_ht_build_kv", "sdb_probe_full", "sdb_compact_row_ids",
              "sdb_gather_i32", "sdb_count_flags", "sdb_fused_chain", "sdb_engine_execute", "sdb_last_error"]:
        assert k in names


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the bindings cover every declaration
    assert set(declared_functions()) <= set(capi.exported_symbols())


def test_abi_struct_sizes():
    L = capi.lib()  # lib() itself raises on a mismatch
    assert L.sdb_abi_sizeof(b"sdb_chain_desc") == ctypes.sizeof(capi.ChainDesc)
    assert L.sdb_abi_sizeof(b"nope") == 0
    assert L.sdb_version().startswith(b"sycldb-gb300")


def test_generator_is_deterministic_and_in_range():
    L = capi.lib()
    a = np.empty(100_003, np.int32)
    b = np.empty(100_003, np.int32)
    capi.check(L.sdb_gen_uniform_cpu(a.ctypes.data, a.size, 0, 7, 3, 90_000, 10_494_950))
    capi.check(L.sdb_gen_uniform_cpu(b.ctypes.data, 50, 100_003 - 50, 7, 3, 90_000, 10_494_950))
    assert np.array_equal(a[-50:], b[:50])  # any row range gives the same values
    assert a.min() >= 90_000 and a.max() <= 10_494_950
    assert L.sdb_gen_uniform_host(7, 3, 12345, 90_000, 10_494_950) == a[12345]
    # roughly uniform
    assert abs(a.mean() - (90_000 + 10_494_950) / 2) < 0.01 * 10_494_950


def test_dates_cover_the_calendar():
    d = ssb.gen_ddate()
    assert d[0][0] == 19920101 and d[0][-1] == 19981230 and d[0].size == 2556
    assert d[4].min() == 1992 and d[4].max() == 1998
    assert d[10].min() == 1 and d[10].max() == 12 and d[11].max() == 53
    f = ssb.gen_lineorder_host(200_000, [5], 1.0)[5]
    assert set(np.unique(f)) <= set(d[0].tolist())


def test_plan_check_orders_and_rejects():
    L = capi.lib()
    p = json.dumps(plans.plan_star(1, 1))
    n = ctypes.c_int()
    order = (ctypes.c_int * 32)()
    capi.check(L.sdb_plan_check(p.encode(), ctypes.byref(n), order, 32))
    assert n.value == 12
    assert list(order[:n.value]) == [1, 4, 7, 2, 5, 0, 3, 6, 8, 9, 10, 11]
    for bad in ['{"rels": [', '{"nope": []}', '{"rels": [{"id": 0, "relOp": "SCAN"}]}',
                '{"rels": [{"id": 0, "relOp": "TABLE_SCAN", "tables": ["ssb", "nosuch"]}]}',
                '{"rels": [{"id": 1, "relOp": "TABLE_SCAN", "tables": ["ssb", "part"]}]}']:
        assert L.sdb_plan_check(bad.encode(), None, None, 0) == capi.SDB_ERR_INVALID
        assert capi.last_error()


def test_plan_check_numeric_enums():
    """Enums may be given by IDL number (TABLE_SCAN=0, FILTER=1, ..., COLUMN=1)."""
    p = {"rels": [{"id": 0, "relOp": 0, "tables": ["ssb", "lineorder"]},
                  {"id": 1, "relOp": 1, "condition": {"exprType": 2, "op": "<", "operands": [
                      {"exprType": 1, "input": 8}, {"exprType": 0, "literal": {"literalOption": 0, "value": 25}}]}},
                  {"id": 2, "relOp": 4, "group": [], "aggs": [{"agg": "SUM", "operands": [9]}]}]}
    n = ctypes.c_int()
    capi.check(capi.lib().sdb_plan_check(json.dumps(p).encode(), ctypes.byref(n), None, 0))
    assert n.value == 3


def test_argument_errors_need_no_device():
    L = capi.lib()
    assert L.sdb_fused_chain(None, None) == capi.SDB_ERR_INVALID
    d = capi.ChainDesc()
    d.n_ops = capi.CHAIN_MAX_OPS + 1
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID
    d.n_ops = 1
    d.ops[0].kind = 99
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID
    assert "unknown op" in capi.last_error()
    d.ops[0].kind = capi.OP_FULL_PROBE
    d.ops[0].a.kind = capi.SRC_LIT
    d.ops[0].ht = None
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID
    assert L.sdb_groupby_sum(None, None, None, 0, None, None, 10, 5, None, None, None, None) == capi.SDB_ERR_INVALID
    assert L.sdb_select_lit(None, 1, 0, 0, None, None, 10, None) == capi.SDB_ERR_INVALID
    assert L.sdb_binop_cc(None, None, None, 9, None, 10, None) == capi.SDB_ERR_INVALID
    assert L.sdb_compact_row_ids(None, 10, None, None, None, 0, None) == capi.SDB_ERR_INVALID
    assert L.sdb_gen_uniform_cpu(None, 0, 0, 1, 1, 5, 4) == capi.SDB_ERR_INVALID
    assert L.sdb_compact_scratch_bytes(0) == 0
    assert L.sdb_compact_scratch_bytes(1) == 256


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(capi, "_LIB", None)
    monkeypatch.setattr(capi, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(RuntimeError, match="not built"):
        capi.lib()


def test_misaligned_typed_pointers_are_rejected_on_the_host():
    """A typed device access at a misaligned address would fault the GPU, so
    the entry points refuse such pointers before launching anything."""
    L = capi.lib()
    odd = 0x1001  # never dereferenced: the check comes first
    assert L.sdb_select_lit(odd, 1, 0, 0, 0x2000, 0x3000, 10, None) == capi.SDB_ERR_INVALID
    assert "aligned" in capi.last_error()
    assert L.sdb_sum_i32_u64(0x2000, 0x3000, 10, 0x4004, None) == capi.SDB_ERR_INVALID
    assert L.sdb_probe_full(0x2000, 0x3002, 0x1, 0x2, 10, 0x4000, 0, 5, None) == capi.SDB_ERR_INVALID
    assert L.sdb_gather_u64(0x2004, 0x3000, 0x4000, 0x5000, 10, None) == capi.SDB_ERR_INVALID
    d = capi.ChainDesc()
    d.n = 10
    d.n_ops = 1
    d.ops[0].kind = capi.OP_SELECT
    d.ops[0].a.kind = capi.SRC_COL
    d.ops[0].a.col = odd
    d.ops[0].b.kind = capi.SRC_LIT
    d.terminal = capi.TERM_FLAGS
    d.flags_out = 0x2000
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID


def test_build_chain_checks_need_no_device():
    """Build terminals are checked on the host; a chain batch refuses a build
    chain that probes a table another build chain of the batch writes (all
    builds share one launch)."""
    L = capi.lib()

    def build(ht, probe_ht=None):
        d = capi.ChainDesc()
        d.n = 1000
        d.terminal = capi.TERM_BUILD_KV
        d.build_key.kind = capi.SRC_COL
        d.build_key.col = 0x10000
        d.build_val.kind = capi.SRC_COL
        d.build_val.col = 0x20000
        d.ht_out = ht
        d.ht_min = 1
        d.ht_len = 1000
        if probe_ht:
            d.n_ops = 1
            d.ops[0].kind = capi.OP_SEMI_PROBE
            d.ops[0].a.kind = capi.SRC_COL
            d.ops[0].a.col = 0x30000
            d.ops[0].lo, d.ops[0].hi = 0, 99
            d.ops[0].ht = probe_ht
        return d

    d = build(0)
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID
    assert "ht_out" in capi.last_error()
    d = build(0x40004)  # a key/value table must be 8-byte aligned
    assert L.sdb_fused_chain(ctypes.byref(d), None) == capi.SDB_ERR_INVALID
    ok = (capi.ChainDesc * 2)(build(0x40000), build(0x50000, probe_ht=0x60000))
    assert L.sdb_chain_batch_scratch_bytes(ok, 2) > 0
    bad = (capi.ChainDesc * 2)(build(0x40000), build(0x50000, probe_ht=0x40000))
    assert L.sdb_chain_batch_scratch_bytes(bad, 2) == 0
    h = ctypes.c_void_p()
    assert L.sdb_chain_batch_create(bad, 2, 0x100000, 1 << 20, None, ctypes.byref(h)) == capi.SDB_ERR_INVALID
    assert "built in the same batch" in capi.last_error()


def test_chain_specialised_is_a_host_query():
    """sdb_chain_specialised: 1 for a chain with a shape-specialised pass, 0
    for one only the general pass runs, a negative status when invalid."""
    L = capi.lib()

    def semi(o, col, ht):
        o.kind = capi.OP_SEMI_PROBE
        o.a.kind = capi.SRC_COL
        o.a.col = col
        o.lo, o.hi, o.ht = 1, 1000, ht

    d = capi.ChainDesc()
    d.n = 1000
    d.n_ops = 2
    semi(d.ops[0], 0x10000, 0x20000)
    semi(d.ops[1], 0x30000, 0x40000)
    d.terminal = capi.TERM_FLAGS
    d.flags_out = 0x50000
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d.n_ops = 1  # one semi probe alone: no specialised shape
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 0
    d.n_ops = 2
    d.flags_out = 0  # a flags chain without flags_out is invalid
    assert L.sdb_chain_specialised(ctypes.byref(d)) == capi.SDB_ERR_INVALID


def _col(o, addr):
    o.kind = capi.SRC_COL
    o.col = addr


def _reg(o, r):
    o.kind = capi.SRC_REG
    o.reg = r


def _star_desc(keys=(1, 0)):
    """The star-join chain as the executor's fuser emits it: semi probe on
    suppkey; full probes on partkey (-> r0) and orderdate (-> r1); group by
    (r1, r0) summing revenue."""
    d = capi.ChainDesc()
    d.n = 1 << 20
    d.n_ops = 3
    o = d.ops[0]
    o.kind, o.lo, o.hi, o.ht = capi.OP_SEMI_PROBE, 1, 40000, 0x200000
    _col(o.a, 0x10000000)
    for i, (col, ht, reg) in enumerate(((0x20000000, 0x300000, 0), (0x30000000, 0x400000, 1)), start=1):
        o = d.ops[i]
        o.kind, o.lo, o.hi, o.ht, o.out_reg = capi.OP_FULL_PROBE, 1, 1000, ht, reg
        _col(o.a, col)
    d.terminal = capi.TERM_GROUPBY
    _col(d.value, 0x40000000)
    d.n_keys = 2
    for q, r in enumerate(keys):
        _reg(d.keys[q], r)
        d.key_min[q], d.key_max[q] = 0, 99
        d.out_keys[q] = 0x500000 + 0x10000 * q
    d.P, d.out_sum, d.occ = 10000, 0x600000, 0x700000
    return d


def _date_join_desc():
    """Date join: discount range; full probe on orderdate (-> r0); r1 =
    extendedprice * discount; group by r0 summing r1."""
    d = capi.ChainDesc()
    d.n = 1 << 20
    d.n_ops = 3
    o = d.ops[0]
    o.kind, o.lo, o.hi, o.logic_op = capi.OP_SEARCH_RANGE, 4, 6, capi.NONE  # the fuser's first op
    _col(o.a, 0x10000000)
    o = d.ops[1]
    o.kind, o.lo, o.hi, o.ht, o.out_reg = capi.OP_FULL_PROBE, 19920101, 19981230, 0x300000, 0
    _col(o.a, 0x20000000)
    o = d.ops[2]
    o.kind, o.bin_op, o.out_reg = capi.OP_BINOP, capi.MUL, 1
    _col(o.a, 0x30000000)
    _col(o.b, 0x10000000)
    d.terminal = capi.TERM_GROUPBY
    _reg(d.value, 1)
    d.n_keys = 1
    _reg(d.keys[0], 0)
    d.key_min[0], d.key_max[0] = 1992, 1998
    d.out_keys[0] = 0x500000
    d.P, d.out_sum, d.occ = 7, 0x600000, 0x700000
    return d


def _filter_sum_desc():
    """Filter-project-sum: orderdate and discount ranges, quantity < 25;
    r0 = extendedprice * discount; sum r0."""
    d = capi.ChainDesc()
    d.n = 1 << 20
    d.n_ops = 4
    for i, (col, lo, hi) in enumerate(((0x10000000, 19940101, 19941231), (0x20000000, 1, 3))):
        o = d.ops[i]
        o.kind, o.lo, o.hi, o.logic_op = capi.OP_SEARCH_RANGE, lo, hi, capi.AND
        _col(o.a, col)
    o = d.ops[2]
    o.kind, o.cmp_op, o.logic_op = capi.OP_SELECT, capi.LT, capi.AND
    _col(o.a, 0x30000000)
    o.b.kind, o.b.lit = capi.SRC_LIT, 25
    o = d.ops[3]
    o.kind, o.bin_op, o.out_reg = capi.OP_BINOP, capi.MUL, 0
    _col(o.a, 0x40000000)
    _col(o.b, 0x20000000)
    d.terminal = capi.TERM_SUM
    _reg(d.value, 0)
    d.sum_out = 0x600000
    return d


def _flight3_desc():
    """SSB flight 3 as the fuser emits it: full probes on custkey (-> r0),
    suppkey (-> r1) and orderdate (-> r2); group by (r0, r1, r2) summing
    revenue.  The supplier table is the smallest."""
    d = capi.ChainDesc()
    d.n = 1 << 20
    d.n_ops = 3
    for i, (col, lo, hi, ht) in enumerate(((0x10000000, 1, 600000, 0x1000000), (0x20000000, 1, 40000, 0x2000000),
                                           (0x30000000, 19920101, 19981230, 0x3000000))):
        o = d.ops[i]
        o.kind, o.lo, o.hi, o.ht, o.out_reg = capi.OP_FULL_PROBE, lo, hi, ht, i
        _col(o.a, col)
    d.terminal = capi.TERM_GROUPBY
    _col(d.value, 0x40000000)
    d.n_keys = 3
    for q in range(3):
        _reg(d.keys[q], q)
        d.key_min[q], d.key_max[q] = 0, 30
        d.out_keys[q] = 0x500000 + 0x10000 * q
    d.P, d.out_sum, d.occ = 31 * 31 * 31, 0x600000, 0x700000
    return d


def _flight4b_desc():
    """Flight 4's second pass as the fuser's split emits it: the rows that
    passed the supplier and part semi joins arrive as flags; full probes on
    custkey (-> r0) and orderdate (-> r1); r2 = revenue - supplycost; group
    by (r1, r0) summing r2."""
    d = capi.ChainDesc()
    d.n = 1 << 20
    d.flags_in = 0x800000
    d.n_ops = 3
    for i, (col, lo, hi, ht) in enumerate(((0x10000000, 1, 600000, 0x1000000),
                                           (0x20000000, 19920101, 19981230, 0x3000000))):
        o = d.ops[i]
        o.kind, o.lo, o.hi, o.ht, o.out_reg = capi.OP_FULL_PROBE, lo, hi, ht, i
        _col(o.a, col)
    o = d.ops[2]
    o.kind, o.bin_op, o.out_reg = capi.OP_BINOP, capi.SUB, 2
    _col(o.a, 0x30000000)
    _col(o.b, 0x40000000)
    d.terminal = capi.TERM_GROUPBY
    _reg(d.value, 2)
    d.n_keys = 2
    for q, r in enumerate((1, 0)):
        _reg(d.keys[q], r)
        d.key_min[q], d.key_max[q] = 0, 30
        d.out_keys[q] = 0x500000 + 0x10000 * q
    d.P, d.out_sum, d.occ = 31 * 31, 0x600000, 0x700000
    return d


def test_hot_shapes_take_their_bound_pass():
    """The star join, date join and filter-project-sum chains in the form
    the fuser emits map to their bound pass (2); an operand elsewhere (the
    star's group keys swapped, a column in place of the select's literal)
    keeps the shape's run-time-bound pass (1)."""
    L = capi.lib()
    for d in (_star_desc(), _date_join_desc(), _filter_sum_desc(), _flight3_desc(), _flight4b_desc()):
        assert L.sdb_chain_specialised(ctypes.byref(d)) == 2
    d = _flight4b_desc()  # without incoming flags nothing to compact on before the first probe
    d.flags_in = 0
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d = _flight3_desc()  # every table too large for a bitmap: no pre-test, no compaction
    d.ops[1].hi = 1 << 20
    d.ops[2].lo, d.ops[2].hi = 0, 1 << 20
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d = _flight3_desc()  # the supplier table 8-byte aligned only: no bitmap from it, the date table instead
    d.ops[1].ht = 0x2000008
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d = _star_desc(keys=(0, 1))
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d = _filter_sum_desc()
    _col(d.ops[2].b, 0x10000000)  # quantity < orderdate
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1
    d = _star_desc()
    d.n = 1 << 31  # row numbers past 31 bits: no late columns, no bound pass
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 1


def test_shared_scans_pair_only_chains_of_one_pass_over_the_same_staged_columns():
    """sdb_chain_pairable: two chains share a paired pass when the
    single-chain pass would run both as the same bound variant-8
    instantiation over the same staged columns and rows; their tables,
    literals, late columns and outputs may differ."""
    L = capi.lib()
    keys = [(capi.TERM_GROUPBY, 2, capi.OP_SEMI_PROBE), (capi.TERM_GROUPBY, 2, capi.OP_SEARCH_RANGE),
            (capi.TERM_SUM, 2, capi.OP_SEARCH_RANGE), (capi.TERM_GROUPBY, 4, capi.OP_FULL_PROBE)]
    rows = 1 << 20
    saved = [L.sdb_chain_tune_get_op(t, r, k, rows) for t, r, k in keys]

    def pairable(a, b):
        return L.sdb_chain_pairable(ctypes.byref(a), ctypes.byref(b))

    def other_star():
        d = _star_desc()
        d.ops[0].ht, d.ops[0].lo, d.ops[0].hi = 0x210000, 1, 30000  # another supplier table and range
        d.ops[1].ht, d.ops[2].ht = 0x310000, 0x410000
        d.out_keys[0], d.out_keys[1], d.out_sum, d.occ = 0x800000, 0x810000, 0x820000, 0x830000
        return d

    try:
        for t, r, k in keys:
            assert L.sdb_chain_tune_set_op(t, r, k, rows, 8) == capi.SDB_OK
        assert pairable(_star_desc(), other_star()) == 1

        def key(d):
            k = ctypes.c_uint64()
            return k.value if L.sdb_chain_pair_key(ctypes.byref(d), ctypes.byref(k)) == 1 else None

        assert key(_star_desc()) is not None and key(_star_desc()) == key(other_star())
        assert len({key(_star_desc()), key(_date_join_desc()), key(_filter_sum_desc())}) == 3
        assert key(_flight3_desc()) is None
        assert pairable(_date_join_desc(), _date_join_desc()) == 1
        assert pairable(_filter_sum_desc(), _filter_sum_desc()) == 1
        d = other_star()
        _col(d.value, 0x41000000)  # revenue of another table: a late column, each chain's own
        _col(d.ops[2].a, 0x31000000)  # orderdate too
        assert pairable(_star_desc(), d) == 1
        d = other_star()
        _col(d.ops[1].a, 0x21000000)  # partkey is staged: not the same columns
        assert pairable(_star_desc(), d) == 0
        d = other_star()
        d.n = (1 << 20) - 1  # other rows
        assert pairable(_star_desc(), d) == 0
        d = other_star()
        d.flags_in = 0x900000  # incoming flags
        assert pairable(_star_desc(), d) == 0
        assert pairable(_star_desc(), _date_join_desc()) == 0  # two shapes
        assert pairable(_star_desc(), _star_desc(keys=(0, 1))) == 0  # the run-time-bound pass
        assert pairable(_flight3_desc(), _flight3_desc()) == 0  # a bound shape without a paired pass
        # a launch of chains that cannot pair is refused on the host, before any device work
        st = L.sdb_chain_launch_pair(ctypes.byref(_star_desc()), ctypes.byref(_date_join_desc()), None)
        assert st == capi.SDB_ERR_UNSUPPORTED and "paired pass" in capi.last_error()
        assert L.sdb_chain_launch_pair(None, ctypes.byref(_star_desc()), None) == capi.SDB_ERR_INVALID
        L.sdb_chain_tune_set_op(capi.TERM_GROUPBY, 2, capi.OP_SEMI_PROBE, rows, 7)
        assert pairable(_star_desc(), other_star()) == 0  # only variant 8 pairs
    finally:
        for (t, r, k), v in zip(keys, saved):
            L.sdb_chain_tune_set_op(t, r, k, rows, v)


def test_plan_order_matches_the_oracle_for_every_shape():
    """The engine's DAG order (operations/preprocessing.cpp:14-102, lineorder
    scans deferred) equals the oracle restatement's for every plan builder."""
    from oracle import oracle as O

    L = capi.lib()
    shapes = [plans.plan_filter_sum(1994), plans.plan_date_join(1995), plans.plan_star(2, 11),
              plans.plan_star(1, 3, 1993, 1996, 12), plans.plan_customer_supplier_date(2),
              plans.plan_customer_supplier_date(0, 1992, 1998, city_points=(21, 27)),
              plans.plan_profit(1), plans.plan_profit(3, (2, 4))]
    for p in shapes:
        n = ctypes.c_int()
        order = (ctypes.c_int * 64)()
        capi.check(L.sdb_plan_check(json.dumps(p).encode(), ctypes.byref(n), order, 64))
        assert list(order[:n.value]) == O.dag_topological_sort(p["rels"]), json.dumps(p)


def test_plan_check_rejects_malformed_graphs():
    """A FILTER with no node before it, a JOIN without two inputs or with an
    input out of range: the plan is refused on the host, with a message."""
    L = capi.lib()
    scan = {"id": 0, "relOp": "TABLE_SCAN", "tables": ["ssb", "part"]}
    bad = [
        {"rels": [{"id": 0, "relOp": "FILTER", "condition": {"exprType": "LITERAL"}}]},
        {"rels": [scan, {"id": 1, "relOp": "JOIN", "inputs": [0], "joinType": "inner",
                         "condition": {"exprType": "EXPR", "op": "=", "operands": []}}]},
        {"rels": [scan, {"id": 1, "relOp": "JOIN", "inputs": [0, 7], "joinType": "inner",
                         "condition": {"exprType": "EXPR", "op": "=", "operands": []}}]},
    ]
    for p in bad:
        assert L.sdb_plan_check(json.dumps(p).encode(), None, None, 0) == capi.SDB_ERR_INVALID, json.dumps(p)
        assert capi.last_error()


def test_open_addressing_entries_check_on_the_host():
    """sdb_oa_log2_slots sizes a table at least twice the build rows; the
    open-addressing entries and chain ops refuse bad slot counts, key ranges
    and alignment before touching a device."""
    L = capi.lib()
    assert L.sdb_oa_log2_slots(0) == 4
    assert L.sdb_oa_log2_slots(8) == 4
    assert L.sdb_oa_log2_slots(9) == 5
    assert L.sdb_oa_log2_slots(1 << 20) == 21
    assert L.sdb_oa_log2_slots((1 << 30) + 1) == capi.SDB_ERR_INVALID
    assert L.sdb_probe_semi_oa(None, None, None, 0, None, 0, 1, 10, None) == capi.SDB_ERR_INVALID
    assert L.sdb_probe_semi_oa(None, None, None, 0, None, 32, 1, 10, None) == capi.SDB_ERR_INVALID
    assert L.sdb_probe_semi_oa(None, None, None, 0, None, 8, 10, 1, None) == capi.SDB_ERR_INVALID  # empty range
    assert L.sdb_probe_full_oa(None, None, None, None, 0, None, 8, -(1 << 31), (1 << 31) - 1, None) == \
        capi.SDB_ERR_INVALID  # 2^32 keys
    assert L.sdb_probe_full_oa(None, None, None, None, 0, 0x1004, 8, 1, 10, None) == capi.SDB_ERR_INVALID  # align
    assert L.sdb_ht_build_kv_oa(None, None, None, 0, 0x1000, 8, 1, 10, 1, None) == capi.SDB_OK
    d = _star_desc()
    d.ops[1].ht_log2 = 40
    assert L.sdb_chain_registers(ctypes.byref(d)) == capi.SDB_ERR_INVALID
    d.ops[1].ht_log2 = 12
    assert L.sdb_chain_registers(ctypes.byref(d)) == 2
    assert L.sdb_chain_specialised(ctypes.byref(d)) == 0  # open-addressing probes: the general pass
