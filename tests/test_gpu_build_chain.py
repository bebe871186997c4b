"""Hash-table builds as fused-chain terminals (SDB_TERM_BUILD_KEYS / _KV): a
dimension's filter ops and its K10 / K12 build in one pass, alone and in a
chain batch's build launch, against the oracle's select + build sequence."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from sycldb_gb300 import capi
from tests import kernel_cases as kc
from tests.gpu_util import dev, host, stream, zeros

pytestmark = pytest.mark.gpu

GE, LE, LT = 5, 3, 2  # comp_op codes used below (EQ..GE = 0..5: EQ NE LT LE GT GE)
NONE, AND = 0, 1


def col(op, ptr):
    op.kind = capi.SRC_COL
    op.col = ptr


def lit(op, v):
    op.kind = capi.SRC_LIT
    op.lit = v


class Dim:
    """A dimension segment: unique keys in [mn, mn + length) (a shuffled
    sample, so some slots have no row), a filter column, a value column and
    input flags; tables pre-filled with a marker so untouched slots show."""

    def __init__(self, n, seed, spare=0.25):
        rng = np.random.default_rng(seed)
        self.n = n
        self.mn = int(rng.integers(-1000, 1000))
        self.length = max(1, int(n * (1 + spare)))
        self.key = (rng.permutation(self.length)[:n] + self.mn).astype(np.int32)
        self.a = rng.integers(0, 100, n).astype(np.int32)
        self.val = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
        self.fin = kc.flags(rng, n, 0.7, canonical=False)
        self.keep = []
        self.p_key = self._dev(self.key)
        self.p_a = self._dev(self.a)
        self.p_val = self._dev(self.val)
        self.p_fin = self._dev(self.fin)

    def _dev(self, x):
        b, p = dev(x if x.size else np.zeros(1, x.dtype))
        self.keep.append(b)
        return p

    def table(self, kv, fill=7):
        init = np.full(2 * self.length if kv else self.length, fill, np.int32 if kv else np.uint8)
        b, p = dev(init)
        self.keep.append(b)
        return b, p, init


def expected(dim, kv, flags, vals=None, fill=7):
    """The oracle's K10 / K12 with the chain's final flags over a pre-filled table."""
    ht = np.full(2 * dim.length if kv else dim.length, fill, np.int32 if kv else np.uint8)
    if kv:
        O.ht_build_kv(dim.key, dim.val if vals is None else vals, flags, ht, dim.mn, dim.length)
    else:
        O.ht_build_keys(dim.key, flags, ht, dim.mn, dim.length)
    return ht


def build_desc(dim, kv, ht_ptr, shape):
    d = capi.ChainDesc()
    d.n = dim.n
    d.terminal = capi.TERM_BUILD_KV if kv else capi.TERM_BUILD_KEYS
    col(d.build_key, dim.p_key)
    col(d.build_val, dim.p_val)
    d.ht_out = ht_ptr
    d.ht_min = dim.mn
    d.ht_len = dim.length
    if shape == "select":  # a < 40, logic NONE (overwrites the input flags)
        d.n_ops = 1
        o = d.ops[0]
        o.kind = capi.OP_SELECT
        o.cmp_op, o.logic_op = LT, NONE
        col(o.a, dim.p_a)
        lit(o.b, 40)
        flags = (dim.a < 40).astype(np.uint8)
    elif shape == "flags_search":  # flags_in AND 10 <= a <= 70
        d.flags_in = dim.p_fin
        d.n_ops = 1
        o = d.ops[0]
        o.kind = capi.OP_SEARCH_RANGE
        o.logic_op = AND
        col(o.a, dim.p_a)
        o.lo, o.hi = 10, 70
        flags = ((dim.fin != 0) & (dim.a >= 10) & (dim.a <= 70)).astype(np.uint8)
    elif shape == "all":  # no op, every row live
        flags = np.ones(dim.n, np.uint8)
    else:
        raise ValueError(shape)
    return d, flags


@pytest.mark.parametrize("n", [1, 255, 1024, 1025, 70_001])
@pytest.mark.parametrize("kv", [False, True])
@pytest.mark.parametrize("shape", ["select", "flags_search", "all"])
@pytest.mark.parametrize("zeroed", [False, True])
def test_build_chain_equals_select_then_build(n, kv, shape, zeroed):
    """zeroed: the table starts all zero and the chain is told so (dead rows
    are not written); otherwise it starts as a marker and every row writes."""
    dim = Dim(n, seed=n * 7 + kv)
    fill = 0 if zeroed else 7
    hb, hp, _ = dim.table(kv, fill)
    d, flags = build_desc(dim, kv, hp, shape)
    d.ht_zeroed = int(zeroed)
    capi.check(capi.lib().sdb_fused_chain(ctypes.byref(d), stream()))
    want = expected(dim, kv, flags, fill=fill)
    got = host(hb, hp, want.size, want.dtype)
    assert np.array_equal(got, want)


def test_build_value_from_a_register_and_flags_out():
    """build_val from an in-chain projection (BINOP a * 3) and the final flags
    also stored: the composed K5 + K12 sequence."""
    dim = Dim(5000, seed=3)
    hb, hp, _ = dim.table(True)
    fb, fp = zeros(dim.n, np.uint8)
    d, flags = build_desc(dim, True, hp, "select")
    o = d.ops[1]
    o.kind = capi.OP_BINOP
    o.bin_op = 0  # Mul
    col(o.a, dim.p_a)
    lit(o.b, 3)
    o.out_reg = 0
    d.n_ops = 2
    d.build_val.kind = capi.SRC_REG
    d.build_val.reg = 0
    d.flags_out = fp
    capi.check(capi.lib().sdb_fused_chain(ctypes.byref(d), stream()))
    want = expected(dim, True, flags, vals=(dim.a * 3).astype(np.int32))
    assert np.array_equal(host(hb, hp, want.size, np.int32), want)
    assert np.array_equal(host(fb, fp, dim.n, np.uint8), flags)


def test_out_of_range_build_keys_are_counted():
    L = capi.lib()
    cnt = ctypes.c_uint64()
    capi.check(L.sdb_device_errors(ctypes.byref(cnt), stream()))  # clear
    dim = Dim(300, seed=9)
    dim.key[5] = dim.mn - 1  # (-1) % len < 0: counted, skipped
    _, dim.p_key = dev(dim.key)
    hb, hp, _ = dim.table(False)
    d, flags = build_desc(dim, False, hp, "all")
    capi.check(L.sdb_fused_chain(ctypes.byref(d), stream()))
    want = np.full(dim.length, 7, np.uint8)
    ok = np.arange(dim.n) != 5
    want[dim.key[ok] - dim.mn] = 1
    assert np.array_equal(host(hb, hp, dim.length, np.uint8), want)
    capi.check(L.sdb_device_errors(ctypes.byref(cnt), stream()))
    assert cnt.value == 1


def probe_sum_desc(n, p_fk1, p_fk2, p_val, d1, ht1, d2, ht2, sum_ptr):
    """Fact chain: semi probe of table 1, full probe of table 2 into reg 0,
    SUM of val over surviving rows."""
    d = capi.ChainDesc()
    d.n = n
    d.n_ops = 2
    o = d.ops[0]
    o.kind = capi.OP_SEMI_PROBE
    col(o.a, p_fk1)
    o.lo, o.hi, o.ht = d1.mn, d1.mn + d1.length - 1, ht1
    o = d.ops[1]
    o.kind = capi.OP_FULL_PROBE
    col(o.a, p_fk2)
    o.lo, o.hi, o.ht, o.out_reg = d2.mn, d2.mn + d2.length - 1, ht2, 0
    d.terminal = capi.TERM_SUM
    col(d.value, p_val)
    d.sum_out = sum_ptr
    return d


@pytest.mark.parametrize("nplans", [1, 5])
def test_batch_builds_run_before_the_chains_that_probe_them(nplans):
    """A chain batch of nplans x (two dimension builds + a fact chain probing
    both): equal to launching every chain on its own, builds first."""
    L = capi.lib()
    rng = np.random.default_rng(nplans)
    keep, chains, tables, sums = [], [], [], []
    want_tables, want_sums = [], []
    for p in range(nplans):
        d1, d2 = Dim(3000 + 17 * p, seed=100 + p), Dim(40_000 + p, seed=200 + p)
        keep += [d1, d2]
        b1, h1, _ = d1.table(False)
        b2, h2, _ = d2.table(True)
        c1, f1 = build_desc(d1, False, h1, "select")
        c2, f2 = build_desc(d2, True, h2, "flags_search")
        nf = 200_000 + 999 * p
        fk1 = rng.integers(d1.mn - 5, d1.mn + d1.length + 5, nf).astype(np.int32)
        fk2 = rng.integers(d2.mn - 5, d2.mn + d2.length + 5, nf).astype(np.int32)
        val = rng.integers(-1000, 1000, nf).astype(np.int32)
        ptrs = []
        for x in (fk1, fk2, val):
            b, q = dev(x)
            keep.append(b)
            ptrs.append(q)
        sb, sp = zeros(1, np.uint64)
        keep.append(sb)
        chains += [c1, c2, probe_sum_desc(nf, *ptrs, d1, h1, d2, h2, sp)]
        tables.append(((b1, h1, d1.length, np.uint8), (b2, h2, 2 * d2.length, np.int32)))
        sums.append((sb, sp))
        t1, t2 = expected(d1, False, f1), expected(d2, True, f2)
        want_tables.append((t1, t2))
        # probe semantics of K13/K15 over the expected tables
        in1 = (fk1 >= d1.mn) & (fk1 <= d1.mn + d1.length - 1)
        hit1 = np.zeros(nf, bool)
        hit1[in1] = t1[fk1[in1] - d1.mn] != 0
        in2 = (fk2 >= d2.mn) & (fk2 <= d2.mn + d2.length - 1)
        hit2 = np.zeros(nf, bool)
        hit2[in2] = t2[2 * (fk2[in2] - d2.mn)] == 1
        live = hit1 & hit2
        want_sums.append(int(val[live].astype(np.int64).astype(np.uint64).sum(dtype=np.uint64)))
    arr = (capi.ChainDesc * len(chains))(*chains)
    nbytes = L.sdb_chain_batch_scratch_bytes(arr, len(chains))
    assert nbytes > 0
    scb, scr = zeros(nbytes + 256, np.uint8)
    scr = (scr + 255) // 256 * 256
    h = ctypes.c_void_p()
    capi.check(L.sdb_chain_batch_create(arr, len(chains), scr, nbytes, stream(), ctypes.byref(h)))
    try:
        assert L.sdb_chain_batch_kernels(h) >= 2  # the build launch + the fact chains
        capi.check(L.sdb_chain_batch_launch(h, stream()))
    finally:
        L.sdb_chain_batch_destroy(h)
    for p in range(nplans):
        for (b, q, n, dt), w in zip(tables[p], want_tables[p]):
            assert np.array_equal(host(b, q, n, dt), w)
        sb, sp = sums[p]
        assert int(host(sb, sp, 1, np.uint64)[0]) == want_sums[p]


@pytest.mark.parametrize("zeroed", [False, True])
def test_interval_tests_cover_every_comparison(zeroed):
    """Selections against literals at the int32 edges (LT INT_MIN, GT INT_MAX,
    NE, an empty SEARCH range, two SEARCH points, OR) become interval tests:
    the same flags as the comparisons."""
    imin, imax = -2**31, 2**31 - 1
    dim = Dim(9000, seed=21)
    rng = np.random.default_rng(4)
    dim.a = rng.choice(np.array([imin, imin + 1, -1, 0, 1, 50, imax - 1, imax], np.int32), dim.n)
    dim.p_a = dim._dev(dim.a)
    a = dim.a.astype(np.int64)
    cases = [  # (ops as (kind, cmp, logic, lo/lit, hi)), expected flags
        ([("sel", 2, NONE, imin, 0)], a < imin),
        ([("sel", 4, NONE, imax, 0)], a > imax),
        ([("sel", 1, NONE, 0, 0)], a != 0),
        ([("sel", 3, NONE, imin, 0), ("sel", 5, AND, imax, 0)], (a <= imin) & (a >= imax)),
        ([("rng", 0, NONE, 5, 4)], np.zeros(dim.n, bool)),
        ([("pts", 0, NONE, imin, imax)], (a == imin) | (a == imax)),
        ([("sel", 0, NONE, 50, 0), ("rng", 0, 2, -1, 1)], (a == 50) | ((a >= -1) & (a <= 1))),
        ([("sel", 2, NONE, 1, 0), ("sel", 4, AND, -1, 0), ("sel", 1, AND, 0, 0), ("sel", 0, 2, imax, 0)],
         ((a < 1) & (a > -1) & (a != 0)) | (a == imax)),
    ]
    for ops, want_flags in cases:
        hb, hp, _ = dim.table(True, 0 if zeroed else 7)
        d, _ = build_desc(dim, True, hp, "all")
        d.ht_zeroed = int(zeroed)
        d.n_ops = len(ops)
        for i, (kind, cmp, logic, v, w) in enumerate(ops):
            o = d.ops[i]
            col(o.a, dim.p_a)
            o.logic_op = logic
            if kind == "sel":
                o.kind, o.cmp_op = capi.OP_SELECT, cmp
                lit(o.b, v)
            else:
                o.kind = capi.OP_SEARCH_RANGE if kind == "rng" else capi.OP_SEARCH_POINTS
                o.lo, o.hi = v, w
        capi.check(capi.lib().sdb_fused_chain(ctypes.byref(d), stream()))
        want = expected(dim, True, want_flags.astype(np.uint8), fill=0 if zeroed else 7)
        assert np.array_equal(host(hb, hp, want.size, np.int32), want), ops
