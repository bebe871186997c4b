"""Operator kernels (K1-K16) through the C ABI on the GPU, against the golden
vectors of the reference functors and against the oracle."""
import ctypes
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from sycldb_gb300 import capi
from tests import kernel_cases as kc
from tests.gpu_util import dev, host, stream, zeros

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(HERE, "kernels.json")))
ARR = np.load(os.path.join(HERE, "kernels.npz"))


def L():
    return capi.lib()


def inp(case, k):
    return ARR["%s/in/%s" % (case["name"], k)].copy()


def run_gpu(case, pad=0):
    """The C-ABI kernel of a golden case; pad=1 offsets every device pointer
    off the 16-byte boundary (keeping each type's natural alignment)."""
    k, p = case["kernel"], case["params"]
    s = stream()
    keep = []

    def D(a):
        # misaligned for the vector paths, naturally aligned for the type
        off = {1: 3, 4: 4, 8: 8}[a.dtype.itemsize] if pad else 0
        b, q = dev(a, off)
        keep.append(b)
        return b, q

    if k in ("select_lit", "select_cols"):
        n = inp(case, "in").size
        _, fin = D(inp(case, "in"))
        ob, out = D(np.zeros(n, np.uint8))
        if k == "select_lit":
            _, col = D(inp(case, "col"))
            capi.check(L().sdb_select_lit(col, p["v"], p["cmp"], p["logic"], fin, out, n, s))
        else:
            _, a = D(inp(case, "a"))
            _, b = D(inp(case, "b"))
            capi.check(L().sdb_select_cols(a, b, p["cmp"], p["logic"], fin, out, n, s))
        return {"out": host(ob, out, n, np.uint8)}
    if k == "logical":
        n = inp(case, "in").size
        _, fin = D(inp(case, "in"))
        _, loc = D(inp(case, "local"))
        ob, out = D(np.zeros(n, np.uint8))
        capi.check(L().sdb_logical(p["logic"], fin, loc, out, n, s))
        return {"out": host(ob, out, n, np.uint8)}
    if k == "fill_i32":
        n = ARR["%s/out/out" % case["name"]].size
        ob, out = D(np.zeros(n, np.int32))
        capi.check(L().sdb_fill_i32(out, p["v"], n, s))
        return {"out": host(ob, out, n, np.int32)}
    if k.startswith("binop_"):
        mode = k.split("_")[1]
        res0 = inp(case, "res0")
        n = res0.size
        rb, res = D(res0)
        _, a = D(inp(case, "a"))
        _, b = D(inp(case, "b"))
        _, fl = D(inp(case, "flags"))
        if mode == "cc":
            capi.check(L().sdb_binop_cc(res, a, b, p["op"], fl, n, s))
        elif mode == "lc":
            capi.check(L().sdb_binop_lc(res, p["la"], b, p["op"], fl, n, s))
        else:
            capi.check(L().sdb_binop_cl(res, a, p["lb"], p["op"], fl, n, s))
        return {"res": host(rb, res, n, np.int32)}
    if k == "sum":
        col = inp(case, "col")
        _, c = D(col)
        _, fl = D(inp(case, "flags"))
        ab, acc = D(np.array([p["acc0"]], np.uint64))
        capi.check(L().sdb_sum_i32_u64(c, fl, col.size, acc, s))
        return {"acc": host(ab, acc, 1, np.uint64)}
    if k == "groupby":
        g, P = p["g"], p["P"]
        val = inp(case, "val")
        n = val.size
        keys = [D(inp(case, "key%d" % j))[1] for j in range(g)]
        okb = [D(np.zeros(P, np.int32)) for _ in range(g)]
        sb, sm = D(np.zeros(P, np.uint64))
        cb, oc = D(np.zeros(P, np.uint32))
        _, v = D(val)
        _, fl = D(inp(case, "flags"))
        mins = (ctypes.c_int32 * g)(*inp(case, "mins").tolist())
        maxs = (ctypes.c_int32 * g)(*inp(case, "maxs").tolist())
        kp = (ctypes.c_void_p * g)(*keys)
        op = (ctypes.c_void_p * g)(*[q for _, q in okb])
        capi.check(L().sdb_groupby_sum(kp, mins, maxs, g, v, fl, n, P, op, sm, oc, s))
        occ = host(cb, oc, P, np.uint32) != 0
        out = {"sum": host(sb, sm, P, np.uint64), "occ": occ.astype(np.uint8)}
        for j in range(g):
            out["okey%d" % j] = np.where(occ, host(okb[j][0], okb[j][1], P, np.int32), 0).astype(np.int32)
        return out
    if k in ("semi", "full"):
        keys = inp(case, "keys")
        nb = keys.size
        probe = inp(case, "probe")
        m = probe.size
        _, kk = D(keys)
        _, bf = D(inp(case, "bflags"))
        _, pr = D(probe)
        _, fin = D(inp(case, "in"))
        ob, out = D(np.zeros(m, np.uint8))
        lo, hi = p["lo"], p["lo"] + p["len"] - 1
        if k == "semi":
            hb, ht = D(np.zeros(nb, np.uint8))
            capi.check(L().sdb_ht_build_keys(kk, bf, nb, ht, lo, p["len"], s))
            capi.check(L().sdb_probe_semi(pr, fin, out, m, ht, lo, hi, s))
            return {"ht": host(hb, ht, nb, np.uint8), "out": host(ob, out, m, np.uint8)}
        hb, ht = D(np.zeros(2 * nb, np.int32))
        _, vv = D(inp(case, "vals"))
        vb, vo = D(np.full(m, -7, np.int32))
        capi.check(L().sdb_ht_build_kv(kk, vv, bf, nb, ht, lo, p["len"], s))
        capi.check(L().sdb_probe_full(pr, vo, fin, out, m, ht, lo, hi, s))
        return {"ht2": host(hb, ht, 2 * nb, np.int32), "out": host(ob, out, m, np.uint8),
                "val_out": host(vb, vo, m, np.int32)}
    if k == "count":
        f = inp(case, "flags")
        _, fl = D(f)
        cb, c = D(np.zeros(1, np.uint64))
        capi.check(L().sdb_count_flags(fl, f.size, c, s))
        return {"count": host(cb, c, 1, np.uint64)}
    raise KeyError(k)


@pytest.mark.parametrize("pad", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_kernel_matches_reference_golden(case, pad):
    got = run_gpu(case, pad)
    for k in case["outputs"]:
        want = ARR["%s/out/%s" % (case["name"], k)]
        assert np.array_equal(got[k], want), (case["name"], k, pad)


@pytest.mark.parametrize("n", [0] + kc.SIZES + [1 << 20, (1 << 20) + 5])
def test_select_and_sum_vs_oracle(n):
    rng = np.random.default_rng(n + 99)
    col = kc.col_small(rng, n, -50, 50)
    fin = kc.flags(rng, n, 0.6, canonical=False)
    want = np.empty(n, np.uint8)
    O.select_lit(col, 3, O.GT, O.AND, fin, want)
    cb, c = dev(col)
    fb, f = dev(fin)
    ob, o = zeros(n, np.uint8)
    capi.check(capi.lib().sdb_select_lit(c, 3, O.GT, O.AND, f, o, n, stream()))
    assert np.array_equal(host(ob, o, n, np.uint8), want)
    acc = np.zeros(1, np.uint64)
    O.sum_i32_u64(col, fin, acc)
    ab, a = zeros(1, np.uint64)
    capi.check(capi.lib().sdb_sum_i32_u64(c, f, n, a, stream()))
    assert host(ab, a, 1, np.uint64)[0] == acc[0]


def test_division_edge_cases_defined():
    """x/0 -> 0 and INT_MIN/-1 -> INT_MIN (undefined in the reference)."""
    a = np.array([5, -7, kc.I32_MIN, kc.I32_MIN, 9, 0, 12, -12], np.int32)
    b = np.array([0, 0, -1, 1, 2, 0, -5, 5], np.int32)
    fl = np.ones(8, np.uint8)
    want = np.zeros(8, np.int32)
    O.binop_cc(want, a, b, O.DIV, fl)
    assert want.tolist() == [0, 0, kc.I32_MIN, kc.I32_MIN, 4, 0, -2, -2]
    _, pa = dev(a)
    _, pb = dev(b)
    _, pf = dev(fl)
    rb, r = zeros(8, np.int32)
    capi.check(capi.lib().sdb_binop_cc(r, pa, pb, O.DIV, pf, 8, stream()))
    assert np.array_equal(host(rb, r, 8, np.int32), want)


def test_out_of_range_slots_are_counted_not_written():
    L = capi.lib()
    cnt = ctypes.c_uint64()
    capi.check(L.sdb_device_errors(ctypes.byref(cnt), stream()))  # clear
    # HASH = (x - min) % len wraps keys above the range (9 -> slot 2, as in the
    # reference); a key below min gives a negative slot: -4 -> (-5) % 3 = -2.
    keys = np.array([1, 2, -4, 3], np.int32)
    fl = np.ones(4, np.uint8)
    _, k = dev(keys)
    _, f = dev(fl)
    hb, ht = zeros(3, np.uint8)
    capi.check(L.sdb_ht_build_keys(k, f, 4, ht, 1, 3, stream()))
    assert host(hb, ht, 3, np.uint8).tolist() == [1, 1, 1]
    capi.check(L.sdb_device_errors(ctypes.byref(cnt), stream()))
    assert cnt.value == 1


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 4095, 4096, 4097, 100_000, 3 * 4096 * 257 + 11])
@pytest.mark.parametrize("p", [0.0, 0.01, 0.5, 1.0])
def test_compaction_and_gather(n, p):
    rng = np.random.default_rng(n)
    fl = kc.flags(rng, n, p, canonical=False)
    src = rng.integers(-1000, 1000, n).astype(np.int32)
    want = O.compact_row_ids(fl) if n else np.empty(0, np.int32)
    L = capi.lib()
    _, f = dev(fl)
    ib, ids = zeros(max(n, 1), np.int32)
    cb, cnt = zeros(1, np.uint32)
    sbytes = L.sdb_compact_scratch_bytes(n)
    scb, scr = zeros(max(sbytes, 1), np.uint8)
    capi.check(L.sdb_compact_row_ids(f, n, ids, cnt, scr, sbytes, stream()))
    c = int(host(cb, cnt, 1, np.uint32)[0])
    assert c == want.size
    assert np.array_equal(host(ib, ids, c, np.int32), want)
    _, s = dev(src)
    db, d = zeros(max(n, 1), np.int32)
    capi.check(L.sdb_gather_i32(s, ids, cnt, d, n, stream()))
    assert np.array_equal(host(db, d, c, np.int32), src[want])


def test_min_max_and_generator_agree_with_host():
    from sycldb_gb300 import ssb

    L = capi.lib()
    n = 1_000_003
    host_cols = ssb.gen_lineorder_host(n, [5, 9], 20.0, row0=17)
    dev_cols = ssb.gen_lineorder_device(n, [5, 9], 20.0, row0=17)
    for c in (5, 9):
        assert np.array_equal(dev_cols[c].cpu().numpy(), host_cols[c])
        mb, mm = zeros(2, np.int32)
        capi.check(L.sdb_min_max_i32(dev_cols[c].data_ptr(), n, mm, stream()))
        assert host(mb, mm, 2, np.int32).tolist() == list(O.min_max(host_cols[c]))


@pytest.mark.parametrize("n", [0, 1, 1023, 1024, 1025, 7000, 65536])
def test_compact_gather_equals_compaction_then_gathers(n):
    """sdb_compact_gather = sdb_compact_row_ids + one gather per column."""
    rng = np.random.default_rng(n + 5)
    fl = kc.flags(rng, max(n, 1), 0.3, canonical=False)[:n]
    a = rng.integers(-2**31, 2**31 - 1, max(n, 1), dtype=np.int64).astype(np.int32)[:n]
    u = rng.integers(0, 2**63, max(n, 1), dtype=np.uint64)[:n]
    b = rng.integers(-5, 5, max(n, 1)).astype(np.int32)[:n]
    lib = L()
    _, f = dev(fl if n else np.zeros(1, np.uint8))
    srcs = [dev(x if n else np.zeros(1, x.dtype))[1] for x in (a, u, b)]
    outs = [zeros(max(n, 1), x.dtype) for x in (a, u, b)]
    cb, cnt = zeros(1, np.uint32)
    src = (ctypes.c_void_p * 3)(*srcs)
    dst = (ctypes.c_void_p * 3)(*[o[1] for o in outs])
    wide = (ctypes.c_int * 3)(0, 1, 0)
    capi.check(lib.sdb_compact_gather(f, n, 3, src, wide, dst, cnt, stream()))
    c = int(host(cb, cnt, 1, np.uint32)[0])
    sel = np.nonzero(fl)[0]
    assert c == sel.size
    for (buf, ptr), x in zip(outs, (a, u, b)):
        assert np.array_equal(host(buf, ptr, c, x.dtype), x[sel])
    assert lib.sdb_compact_gather(f, 65537, 3, src, wide, dst, cnt, stream()) == capi.SDB_ERR_INVALID


@pytest.mark.parametrize("P_ranges", [(7, 1000), (7, 3000)])  # 7,000 slots (shared table), 21,000 (global)
@pytest.mark.parametrize("n", [1, 17, 4097, 1_000_003])
@pytest.mark.parametrize("pad", [0, 1])
@pytest.mark.parametrize("p", [0.008, 0.6])
def test_groupby_sum_sparse_and_dense_flags_vs_oracle(P_ranges, n, pad, p):
    """K8 over both slot tables (shared memory up to 8192 slots, global
    beyond), with 16-byte aligned and unaligned flags, sparse and dense."""
    rng = np.random.default_rng(n + 31 * P_ranges[1] + pad)
    r0, r1 = P_ranges
    k0 = rng.integers(1992, 1992 + r0, n).astype(np.int32)
    k1 = rng.integers(0, r1, n).astype(np.int32)
    val = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
    fl = kc.flags(rng, n, p, canonical=False)
    P = r0 * r1
    mins = np.array([1992, 0], np.int32)
    maxs = np.array([1992 + r0 - 1, r1 - 1], np.int32)
    want_keys = [np.zeros(P, np.int32), np.zeros(P, np.int32)]
    want_sum = np.zeros(P, np.uint64)
    want_occ = np.zeros(P, np.uint32)
    O.groupby_sum([k0, k1], mins, maxs, val, fl, P, want_keys, want_sum, want_occ)
    lib = L()
    keys = [dev(k)[1] for k in (k0, k1)]
    _, v = dev(val)
    _, f = dev(fl, 1 if pad else 0)  # one byte off: the unaligned flag path
    okb = [zeros(P, np.int32) for _ in range(2)]
    sb, sp = zeros(P, np.uint64)
    ob, op = zeros(P, np.uint32)
    kp = (ctypes.c_void_p * 2)(*keys)
    okp = (ctypes.c_void_p * 2)(*[o[1] for o in okb])
    mn = (ctypes.c_int32 * 2)(*mins.tolist())
    mx = (ctypes.c_int32 * 2)(*maxs.tolist())
    capi.check(lib.sdb_groupby_sum(kp, mn, mx, 2, v, f, n, P, okp, sp, op, stream()))
    occ = host(ob, op, P, np.uint32)
    assert np.array_equal(occ != 0, want_occ != 0)
    assert np.array_equal(host(sb, sp, P, np.uint64), want_sum)
    live = want_occ != 0
    for (b, ptr), w in zip(okb, want_keys):
        assert np.array_equal(host(b, ptr, P, np.int32)[live], w[live])


@pytest.mark.parametrize("n", [0, 1, 1023, 7000, 65536])
def test_compact_gather_occ_equals_occ_to_flags_then_compact_gather(n):
    """sdb_compact_gather_occ = sdb_occ_to_flags + sdb_compact_gather."""
    rng = np.random.default_rng(n + 77)
    m = max(n, 1)
    occ = np.where(rng.random(m) < 0.04, rng.integers(1, 5, m), 0).astype(np.uint32)[:n]
    a = rng.integers(-2**31, 2**31 - 1, m, dtype=np.int64).astype(np.int32)[:n]
    u = rng.integers(0, 2**63, m, dtype=np.uint64)[:n]
    lib = L()
    _, op = dev(occ if n else np.zeros(1, np.uint32))
    srcs = [dev(x if n else np.zeros(1, x.dtype))[1] for x in (a, u)]
    outs = [zeros(m, x.dtype) for x in (a, u)]
    cb, cnt = zeros(1, np.uint32)
    src = (ctypes.c_void_p * 2)(*srcs)
    dst = (ctypes.c_void_p * 2)(*[o[1] for o in outs])
    wide = (ctypes.c_int * 2)(0, 1)
    capi.check(lib.sdb_compact_gather_occ(op, n, 2, src, wide, dst, cnt, stream()))
    c = int(host(cb, cnt, 1, np.uint32)[0])
    sel = np.nonzero(occ)[0]
    assert c == sel.size
    for (buf, ptr), x in zip(outs, (a, u)):
        assert np.array_equal(host(buf, ptr, c, x.dtype), x[sel])


def _force_op_shape(block, per_sm):
    for k in range(len(capi.OP_KERNELS)):
        for b in range(40):
            capi.check(capi.lib().sdb_op_tune_set(k, 1 << b, block, per_sm))


@pytest.mark.parametrize("shape", [(128, 2), (512, 4), (512, 1), (128, 16)])
def test_every_launch_shape_gives_the_golden_vectors(shape):
    """The operator kernels' tuned launch shapes (threads per block x blocks
    per SM) change only how the rows are spread over the grid: every golden
    case, and the oracle sweeps at sizes beyond one wave, give the same."""
    try:
        _force_op_shape(*shape)
        for case in CASES:
            got = run_gpu(case)
            for k in case["outputs"]:
                assert np.array_equal(got[k], ARR["%s/out/%s" % (case["name"], k)]), (case["name"], shape)
        for n in (1000, (1 << 20) + 5, 3 << 20):
            test_select_and_sum_vs_oracle(n)
        test_compaction_and_gather(1 << 20, 0.3)
    finally:
        _force_op_shape(0, 0)
