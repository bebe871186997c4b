"""Open-addressing join tables (sparse key ranges): the K10-K13 forms over
2^lg slots against the direct-address semantics, the executor with every
join on open-addressing tables against the golden results, and a sparse key
range whose direct-address table would not fit the budget."""
import ctypes
import json
import os

import numpy as np
import pytest

from sycldb_gb300 import capi, plans
from sycldb_gb300.engine import Engine
from tests import datasets
from tests.gpu_util import dev, host, release, stream, zeros

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PLANS = json.load(open(os.path.join(HERE, "plans.json")))


def L():
    return capi.lib()


def _load(eng, ds):
    for name, cols in ds.items():
        eng.load_table(name, cols)


def test_oa_builds_and_probes_give_the_direct_table_answers():
    """Two segments of builds (the first into a fresh table, the second
    rewriting keys: live ones with new values, dead ones to misses), then
    probes of present, absent, out-of-range and dead-flag rows: the hits and
    values the direct-address table gives."""
    rng = np.random.default_rng(7)
    mn, mx = -(1 << 29), 1 << 29
    keys = rng.choice(np.arange(mn, mx, 977, dtype=np.int64), 30000, replace=False).astype(np.int32)
    seg1, seg2 = keys[:20000], np.concatenate([keys[10000:15000], keys[20000:]])  # 5000 keys rewritten
    f1 = (rng.random(seg1.size) < 0.6).astype(np.uint8)
    f2 = (rng.random(seg2.size) < 0.5).astype(np.uint8)
    v1 = rng.integers(-(1 << 31), 1 << 31, seg1.size, dtype=np.int64).astype(np.int32)
    v2 = rng.integers(-(1 << 31), 1 << 31, seg2.size, dtype=np.int64).astype(np.int32)
    cnt = ctypes.c_uint64(0)
    capi.check(L().sdb_device_errors(ctypes.byref(cnt), stream()))  # clear
    lg = L().sdb_oa_log2_slots(keys.size)
    assert (1 << lg) >= 2 * keys.size
    # expected: a dict of the direct table's entries after both builds
    want_semi, want_kv = {}, {}
    for k, f in zip(seg1, f1):
        if f:  # fresh table: dead rows' misses are already there
            want_semi[int(k)] = True
    for k, f, v in zip(seg1, f1, v1):
        if f:
            want_kv[int(k)] = int(v)
    for k, f, v in zip(seg2, f2, v2):
        want_semi[int(k)] = bool(f)
        if f:
            want_kv[int(k)] = int(v)
        else:
            want_kv.pop(int(k), None)
    ht_t, ht = zeros(1 << lg, np.uint32)
    kv_t, kv = zeros(2 << lg, np.int32)
    s = stream()
    for seg, f, v, fresh in ((seg1, f1, v1, 1), (seg2, f2, v2, 0)):
        kt, kp = dev(seg)
        ft, fp = dev(f)
        vt, vp = dev(v)
        capi.check(L().sdb_ht_build_keys_oa(kp, fp, seg.size, ht, lg, mn, mx, fresh, s))
        capi.check(L().sdb_ht_build_kv_oa(kp, vp, fp, seg.size, kv, lg, mn, mx, fresh, s))
    probe = np.concatenate([keys, rng.integers(mn, mx, 20000, dtype=np.int64).astype(np.int32),
                            np.array([mn - 1, mx + 1, mn, mx], np.int32)])
    fin = (rng.random(probe.size) < 0.9).astype(np.uint8)
    pt, pp = dev(probe)
    it, ip = dev(fin)
    ot, op = zeros(probe.size, np.uint8)
    o2t, o2 = zeros(probe.size, np.uint8)
    rt, rp = zeros(probe.size, np.int32)
    capi.check(L().sdb_probe_semi_oa(pp, ip, op, probe.size, ht, lg, mn, mx, s))
    capi.check(L().sdb_probe_full_oa(pp, rp, ip, o2, probe.size, kv, lg, mn, mx, s))
    semi = host(ot, op, probe.size, np.uint8)
    full = host(o2t, o2, probe.size, np.uint8)
    res = host(rt, rp, probe.size, np.int32)
    exp_semi = np.array([bool(f) and want_semi.get(int(k), False) for k, f in zip(probe, fin)])
    exp_full = np.array([bool(f) and int(k) in want_kv for k, f in zip(probe, fin)])
    assert np.array_equal(semi.astype(bool), exp_semi)
    assert np.array_equal(full.astype(bool), exp_full)
    hit = np.nonzero(exp_full)[0]
    assert np.array_equal(res[hit], np.array([want_kv[int(probe[i])] for i in hit], np.int32))
    capi.check(L().sdb_device_errors(ctypes.byref(cnt), stream()))
    assert cnt.value == 0
    release()


@pytest.mark.parametrize("fuse", [False, True])
def test_every_join_on_open_addressing_matches_golden(fuse):
    """join_tables = 2: every join of the golden plans (semi and inner, all
    benchmark shapes) on open-addressing tables gives the golden rows."""
    for case in PLANS:
        ds = datasets.dataset(case["sf"], case["seed"])
        with Engine(arena_bytes=1 << 30, fuse=fuse, join_tables=2) as eng:
            _load(eng, ds)
            got = eng.execute(case["plan"]).canonical()
        assert [list(r) for r in got] == case["rows"], case["name"]


def _sparse(ds, supp_stride, part_stride, cust_stride):
    """The dataset with supplier, part and customer keys spread out (fact
    foreign keys scaled alike): the same joins over sparse key ranges."""
    out = {}
    for name, cols in ds.items():
        out[name] = dict(cols)
    def scale(a, k):
        return (a.astype(np.int64) * k).astype(np.int32)
    lo = out["lineorder"]
    lo[4], out["supplier"][0] = scale(lo[4], supp_stride), scale(out["supplier"][0], supp_stride)
    lo[3], out["part"][0] = scale(lo[3], part_stride), scale(out["part"][0], part_stride)
    if "customer" in out:
        lo[2], out["customer"][0] = scale(lo[2], cust_stride), scale(out["customer"][0], cust_stride)
    return out


@pytest.mark.parametrize("fuse", [False, True])
def test_sparse_key_ranges_run_in_budget_and_match_the_oracle(fuse):
    """Supplier keys spread over ~10^8 values: the direct-address semi-join
    table (one byte per key of the range) does not fit a 64 MB budget, the
    default layout picks open addressing for it and the results equal the
    oracle's (direct tables) on the same data."""
    ds = _sparse(datasets.dataset(0.05), 1 << 20, 1009, 1013)
    pls = [plans.plan_star(2, 11), plans.plan_star(1, 3, 1993, 1996, 12),
           plans.plan_customer_supplier_date(1, 1992, 1997)]
    with Engine(arena_bytes=64 << 20, fuse=fuse, join_tables=1) as eng:
        _load(eng, ds)
        with pytest.raises(capi.SdbError) as e:
            eng.execute(pls[0])
        assert e.value.status == capi.SDB_ERR_NOMEM
    with Engine(arena_bytes=64 << 20, fuse=fuse) as eng:
        _load(eng, ds)
        for p in pls:
            assert eng.execute(p).canonical() == datasets.oracle_run(ds, p), json.dumps(p)
