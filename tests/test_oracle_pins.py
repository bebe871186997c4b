"""The oracle's C restatement against the reference's own kernel functors
(kernels/*.hpp compiled here against the host SYCL shim), on seeded inputs.

CPU only.  Skipped where the reference checkout is absent."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests import kernel_cases as kc
from tests import refkern as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference checkout not present")


@pytest.mark.parametrize("n", kc.SIZES)
@pytest.mark.parametrize("cmp", range(6))
@pytest.mark.parametrize("logic", range(3))
def test_select_lit(n, cmp, logic):
    rng = np.random.default_rng(n * 31 + cmp * 7 + logic)
    col = kc.col_small(rng, n)
    fin = kc.flags(rng, n)
    v = int(rng.integers(-5, 6))
    a, b = np.empty(n, np.uint8), np.empty(n, np.uint8)
    O.select_lit(col, v, cmp, logic, fin, a)
    R.lib().ref_select_lit(R.ptr(col), v, cmp, logic, R.ptr(fin), R.ptr(b), n)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("cmp", range(6))
@pytest.mark.parametrize("logic", range(3))
def test_select_cols_wide(cmp, logic):
    rng = np.random.default_rng(100 + cmp * 3 + logic)
    n = 3001
    x, y = kc.col_wide(rng, n), kc.col_wide(rng, n)
    y[::5] = x[::5]
    fin = kc.flags(rng, n)
    a, b = np.empty(n, np.uint8), np.empty(n, np.uint8)
    O.select_cols(x, y, cmp, logic, fin, a)
    R.lib().ref_select_cols(R.ptr(x), R.ptr(y), cmp, logic, R.ptr(fin), R.ptr(b), n)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("op", ["==", "!=", "<>", "<", "<=", ">", ">=", "=", "LIKE", ""])
@pytest.mark.parametrize("parent", ["", "AND", "OR", "NONE", "NOT"])
def test_string_decoding(op, parent):
    """get_comp_op / get_logical_op including the unknown-string defaults."""
    assert O.get_comp_op(op) == R.lib().ref_get_comp_op(op.encode())
    assert O.get_logical_op(parent) == R.lib().ref_get_logical_op(parent.encode())
    rng = np.random.default_rng(5)
    n = 100
    col, fin = kc.col_small(rng, n), kc.flags(rng, n)
    a, b = np.empty(n, np.uint8), np.empty(n, np.uint8)
    O.select_lit(col, 1, O.get_comp_op(op), O.get_logical_op(parent), fin, a)
    R.lib().ref_select_lit_str(R.ptr(col), 1, op.encode(), parent.encode(), R.ptr(fin), R.ptr(b), n)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("op", ["AND", "OR", "SEARCH", ">=", "NOT", "and"])
def test_is_filter_logical(op):
    assert O.is_filter_logical(op) == bool(R.lib().ref_is_filter_logical(op.encode()))


@pytest.mark.parametrize("op", ["*", "/", "+", "-", "%", "x"])
def test_binop_decoding(op):
    r = R.lib().ref_get_binop(op.encode())
    if r < 0:
        with pytest.raises(ValueError):
            O.get_op_from_string(op)
    else:
        assert O.get_op_from_string(op) == r


@pytest.mark.parametrize("logic", range(3))
@pytest.mark.parametrize("n", [1, 33, 1000])
def test_logical(logic, n):
    rng = np.random.default_rng(logic + n)
    fin, loc = kc.flags(rng, n), kc.flags(rng, n)
    a, b = np.empty(n, np.uint8), np.empty(n, np.uint8)
    O.logical(logic, fin, loc, a)
    R.lib().ref_logical(logic, R.ptr(fin), R.ptr(loc), R.ptr(b), n)
    assert np.array_equal(a, b)


def test_fill():
    n = 777
    a, b = np.zeros(n, np.int32), np.zeros(n, np.int32)
    O.fill_i32(a, -12345)
    R.lib().ref_fill_i32(R.ptr(b), -12345, n)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("op", range(4))
@pytest.mark.parametrize("mode", ["cc", "lc", "cl"])
def test_binop(op, mode):
    rng = np.random.default_rng(op * 10 + len(mode))
    n = 2049
    x, y = kc.col_wide(rng, n), kc.col_wide(rng, n)
    lit_a, lit_b = int(kc.col_wide(rng, 1)[0]), int(kc.divisor(rng, 1)[0])
    if op == O.DIV:
        y = kc.divisor(rng, n)
        x = kc.numerators_for(x, y)
        if mode == "lc":
            lit_a = 1 << 30 if lit_a == kc.I32_MIN else lit_a
        if mode == "cl":
            x = kc.numerators_for(x, np.full(n, lit_b, np.int32))
    fl = kc.flags(rng, n)
    a = np.full(n, 99, np.int32)
    b = a.copy()
    if mode == "cc":
        O.binop_cc(a, x, y, op, fl)
        R.lib().ref_binop_cc(R.ptr(b), R.ptr(x), R.ptr(y), op, R.ptr(fl), n)
    elif mode == "lc":
        O.binop_lc(a, lit_a, y, op, fl)
        R.lib().ref_binop_lc(R.ptr(b), lit_a, R.ptr(y), op, R.ptr(fl), n)
    else:
        O.binop_cl(a, x, lit_b, op, fl)
        R.lib().ref_binop_cl(R.ptr(b), R.ptr(x), lit_b, op, R.ptr(fl), n)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("n", kc.SIZES)
def test_sum(n):
    rng = np.random.default_rng(n)
    col = kc.col_wide(rng, n)
    fl = kc.flags(rng, n, 0.7)
    a = np.array([123456789], np.uint64)
    b = a.copy()
    O.sum_i32_u64(col, fl, a)
    R.lib().ref_sum_i32_u64(R.ptr(col), R.ptr(fl), n, R.ptr(b))
    assert a[0] == b[0]


@pytest.mark.parametrize("g", [1, 2, 3])
@pytest.mark.parametrize("n", [1, 100, 5000, 70000])
def test_groupby(g, n):
    rng = np.random.default_rng(g * 1000 + n)
    ranges = [(1992, 1998), (-3, 4), (0, 9)][:g]
    keys = [rng.integers(lo, hi + 1, n).astype(np.int32) for lo, hi in ranges]
    mins = [lo for lo, _ in ranges]
    maxs = [hi for _, hi in ranges]
    P = int(np.prod([hi - lo + 1 for lo, hi in ranges]))
    val = kc.col_wide(rng, n)
    fl = kc.flags(rng, n, 0.6)
    ok = [np.zeros(P, np.int32) for _ in range(g)]
    os_, oc = np.zeros(P, np.uint64), np.zeros(P, np.uint32)
    bad = O.groupby_sum(keys, mins, maxs, val, fl, P, ok, os_, oc)
    assert bad == 0
    rk = [np.zeros(P, np.int32) for _ in range(g)]
    rs, rc = np.zeros(P, np.uint64), np.zeros(P, np.uint32)
    mn, mx = np.array(mins, np.int32), np.array(maxs, np.int32)
    R.lib().ref_groupby_sum(R.ptr_array(keys), R.ptr(mn), R.ptr(mx), g, R.ptr(val), R.ptr(fl), n, P,
                            R.ptr_array(rk), R.ptr(rs), R.ptr(rc))
    assert np.array_equal(os_, rs)
    assert np.array_equal(oc != 0, rc != 0)
    live = rc != 0
    for j in range(g):
        assert np.array_equal(ok[j][live], rk[j][live])


@pytest.mark.parametrize("n", [1, 40, 4000])
def test_semi_join(n):
    rng = np.random.default_rng(n + 7)
    lo = int(rng.integers(-100, 100))
    keys = kc.unique_keys(rng, n, lo)
    bfl = kc.flags(rng, n, 0.3)
    ht1, ht2 = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
    assert O.ht_build_keys(keys, bfl, ht1, lo, n) == 0
    R.lib().ref_ht_build_keys(R.ptr(keys), R.ptr(bfl), n, R.ptr(ht2), lo, n)
    assert np.array_equal(ht1, ht2)
    m = 5 * n + 3
    probe = rng.integers(lo - 3, lo + n + 3, m).astype(np.int32)
    fin = kc.flags(rng, m, 0.8)
    a, b = np.empty(m, np.uint8), np.empty(m, np.uint8)
    O.probe_semi(probe, fin, a, ht1, lo, lo + n - 1)
    R.lib().ref_probe_semi(R.ptr(probe), R.ptr(fin), R.ptr(b), m, R.ptr(ht2), lo, lo + n - 1)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("n", [1, 40, 4000])
def test_full_join(n):
    rng = np.random.default_rng(n + 11)
    lo = int(rng.integers(1, 100))
    keys = kc.unique_keys(rng, n, lo)
    vals = kc.col_wide(rng, n)
    bfl = kc.flags(rng, n, 0.4)
    ht1, ht2 = np.zeros(2 * n, np.int32), np.zeros(2 * n, np.int32)
    assert O.ht_build_kv(keys, vals, bfl, ht1, lo, n) == 0
    R.lib().ref_ht_build_kv(R.ptr(keys), R.ptr(vals), R.ptr(bfl), n, R.ptr(ht2), lo, n)
    assert np.array_equal(ht1, ht2)
    m = 5 * n + 3
    probe = rng.integers(lo - 3, lo + n + 3, m).astype(np.int32)
    fin = kc.flags(rng, m, 0.8)
    a, b = np.empty(m, np.uint8), np.empty(m, np.uint8)
    va, vb = np.full(m, -7, np.int32), np.full(m, -7, np.int32)
    O.probe_full(probe, va, fin, a, ht1, lo, lo + n - 1)
    R.lib().ref_probe_full(R.ptr(probe), R.ptr(vb), R.ptr(fin), R.ptr(b), m, R.ptr(ht2), lo, lo + n - 1)
    assert np.array_equal(a, b)
    assert np.array_equal(va, vb)


@pytest.mark.parametrize("n", [1, 1000, 100001])
def test_count_flags(n):
    rng = np.random.default_rng(n)
    fl = kc.flags(rng, n, 0.3)
    assert O.count_flags(fl) == R.lib().ref_count_flags(R.ptr(fl), n)


@pytest.mark.parametrize("table", ["lineorder", "part", "supplier", "customer", "ddate"])
def test_table_column_maps(table):
    """The loader's column maps (kernels/types.cpp:3-21)."""
    L = R.lib()
    assert O.TABLE_COLUMN_NUMBERS[table] == L.ref_table_column_number(table.encode())
    for c in range(O.TABLE_COLUMN_NUMBERS[table]):
        assert (c in O.TABLE_COLUMN_INDICES[table]) == bool(L.ref_table_column_loaded(table.encode(), c))
