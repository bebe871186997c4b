"""The host executor on the GPU: plans of the benchmark shapes against the
committed golden results and the oracle, operator-at-a-time and fused, with
one and several segments; the SF20 star join at full size."""
import json
import os

import numpy as np
import pytest

from sycldb_gb300 import capi, plans, ssb
from sycldb_gb300.engine import Engine
from tests import datasets, naive

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PLANS = json.load(open(os.path.join(HERE, "plans.json")))


def load(eng, ds, device=False):
    import torch

    for name, cols in ds.items():
        if device:
            eng.load_table(name, {c: torch.from_numpy(a).cuda() for c, a in cols.items()})
        else:
            eng.load_table(name, cols)


@pytest.mark.parametrize("fuse", [False, True])
@pytest.mark.parametrize("seg", [0, 4096])
@pytest.mark.parametrize("case", PLANS, ids=[c["name"] for c in PLANS])
def test_plan_matches_golden(case, fuse, seg):
    ds = datasets.dataset(case["sf"], case["seed"])
    with Engine(arena_bytes=1 << 30, segment_rows=seg, fuse=fuse) as eng:
        load(eng, ds, device=bool(seg))
        got = eng.execute(case["plan"]).canonical()
    assert [list(r) for r in got] == case["rows"]


@pytest.mark.parametrize("fuse", [False, True])
def test_quirk_plans_match_oracle(fuse):
    """Filters with OR / parent-op quirk, SEARCH points, column-column
    comparisons, literal projections, every binary operator."""
    ds = datasets.dataset(0.01)
    P = plans
    cases = []
    b = P.PlanBuilder()
    b.scan("lineorder")
    b.filter(P.AND(P.expr("<=", P.col(8), P.lit(30)),
                   P.OR(P.search_points(11, 2, 7), P.expr(">", P.col(9), P.col(12)))))
    b.project([P.expr("-", P.col(9), P.col(13)), P.lit(3)])
    b.aggregate([], 0)
    cases.append(b.plan())
    for op in ["*", "/", "+", "-"]:
        b = P.PlanBuilder()
        b.scan("lineorder")
        b.filter(P.expr("<>", P.col(11), P.lit(0)))
        b.project([P.col(8), P.expr(op, P.col(9), P.col(11)), P.expr(op, P.lit(1000), P.col(11))])
        b.aggregate([0], 1)
        cases.append(b.plan())
        b = P.PlanBuilder()
        b.scan("lineorder")
        b.project([P.col(11), P.expr(op, P.col(12), P.lit(7))])
        b.aggregate([0], 1)
        cases.append(b.plan())
    b = P.PlanBuilder()  # a plan that ends in a filter (no aggregate)
    b.scan("lineorder")
    b.filter(P.AND(P.expr("==", P.col(11), P.lit(10)), P.expr("<", P.col(8), P.lit(3))))
    b.project([P.col(5), P.col(9)])
    cases.append(b.plan())
    with Engine(arena_bytes=1 << 30, segment_rows=8192, fuse=fuse) as eng:
        load(eng, ds)
        for plan in cases:
            assert eng.execute(plan).canonical() == datasets.oracle_run(ds, plan, 8192), json.dumps(plan)


def test_res_writer(tmp_path):
    ds = datasets.dataset(0.01)
    with Engine(arena_bytes=1 << 30) as eng:
        load(eng, ds)
        plan = plans.plan_date_join(1994)
        p = str(tmp_path / "q.res")
        eng.execute_to_res(plan, p)
        rows = [tuple(int(x) for x in line.split()) for line in open(p).read().splitlines()]
    assert sorted(rows) == datasets.oracle_run(ds, plan)


def test_errors_are_statuses_not_crashes():
    ds = datasets.dataset(0.01)
    with Engine(arena_bytes=1 << 28) as eng:
        load(eng, ds)
        with pytest.raises(capi.SdbError) as e:
            eng.execute('{"rels": [{"id": 0, "relOp": "TABLE_SCAN", "tables": ["ssb", "customerz"]}]}')
        assert e.value.status == capi.SDB_ERR_INVALID
        bad = plans.plan_star(1, 1)
        bad["rels"][3]["condition"]["operands"][1]["input"] = 999
        with pytest.raises(capi.SdbError):
            eng.execute(bad)
        # the engine stays usable
        assert eng.execute(plans.plan_filter_sum(1993)).canonical() == datasets.oracle_run(ds, plans.plan_filter_sum(1993))
    with Engine(arena_bytes=1 << 16) as small:  # budget exceeded -> SDB_ERR_NOMEM
        small.load_table("lineorder", ds["lineorder"])
        with pytest.raises(capi.SdbError) as e:
            small.execute(plans.plan_filter_sum(1993))
        assert e.value.status == capi.SDB_ERR_NOMEM


def test_star_sf20_full_size():
    """The benchmark configuration at full size (120 M fact rows): fused and
    operator-at-a-time results agree and equal the naive evaluator's."""
    import torch

    sf = 20.0
    n = ssb.fact_rows(sf)
    fact = ssb.gen_lineorder_device(n, ssb.QUERY_COLUMNS["star"], sf)
    dims = ssb.gen_dims(sf)
    plan = plans.plan_star(2, 11)
    res = {}
    for fuse in (True, False):
        with Engine(fuse=fuse) as eng:
            eng.load_table("lineorder", fact)
            for t in ("supplier", "part", "ddate"):
                eng.load_table(t, dims[t])
            res[fuse] = eng.execute(plan).canonical()
    assert res[True] == res[False]
    host_fact = {c: t.cpu().numpy() for c, t in fact.items()}
    want = naive.star(host_fact, dims["supplier"], dims["part"], dims["ddate"], 2, 11)
    assert res[True] == want
    assert 200 <= len(want) <= 280
    del fact
    torch.cuda.empty_cache()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5, 6, 7])
def test_every_kernel_variant_matches_golden(variant):
    """The general pass at 4/8/16 rows per thread and the shape-specialised
    pass give the same rows."""
    try:
        capi.force_chain_variant(variant)
        for case in PLANS:
            ds = datasets.dataset(case["sf"], case["seed"])
            with Engine(arena_bytes=1 << 30, fuse=True) as eng:
                load(eng, ds)
                got = eng.execute(case["plan"]).canonical()
            assert [list(r) for r in got] == case["rows"], (variant, case["name"])
    finally:
        capi.force_chain_variant(-1)


@pytest.mark.parametrize("variant", [0, 3, 4, 5, 6, 7, 8])
def test_reversed_search_range_is_empty(variant):
    """A SEARCH range whose low bound is above its high bound selects no row
    (the reference's `c >= lo` then `c <= hi`), in every fused variant."""
    ds = datasets.dataset(0.01)
    P = plans
    b = P.PlanBuilder()
    b.scan("lineorder")
    b.filter(P.AND(P.search(5, 19941231, 19940101), P.search(11, 1, 3), P.expr("<", P.col(8), P.lit(25))))
    b.project([P.expr("*", P.col(9), P.col(11))])
    b.aggregate([], 0)
    rev = b.plan()
    b = P.PlanBuilder()
    f = b.scan("lineorder")
    f = b.filter(P.search(11, 6, 4))
    d = b.scan("ddate")
    d = b.filter(P.search(4, 1993, 1994))
    b.join(f, d, 5, 17)
    b.project([P.col(17 + 4), P.expr("*", P.col(9), P.col(11))])
    b.aggregate([0], 1)
    rev_join = b.plan()
    try:
        capi.force_chain_variant(variant)
        with Engine(arena_bytes=1 << 30, fuse=True) as eng:
            load(eng, ds)
            for plan in (rev, rev_join):
                assert eng.execute(plan).canonical() == datasets.oracle_run(ds, plan), json.dumps(plan)
    finally:
        capi.force_chain_variant(-1)


def test_variant_8_runs_the_hot_shapes_bound():
    """Under variant 8 the star join, date join and filter-project-sum plans
    of the benchmark, as the executor fuses them, run their bound passes
    (every operand at a place fixed at compile time), with the oracle's
    results."""
    ds = datasets.dataset(0.05)
    pls = [plans.plan_star(2, 11), plans.plan_date_join(1995), plans.plan_filter_sum(1994),
           plans.plan_star(1, 3, 1993, 1996, 12), plans.plan_customer_supplier_date(2),
           plans.plan_customer_supplier_date(0, 1993, 1997, (3, 17)), plans.plan_profit(1), plans.plan_profit(3, (2, 4))]
    try:
        with Engine(arena_bytes=1 << 30, fuse=True) as eng:
            capi.force_chain_variant(8)
            load(eng, ds)
            for p in pls:
                before = capi.fused_launch_counts()
                got = eng.execute(p).canonical()
                after = capi.fused_launch_counts()
                assert after[1] - before[1] >= 1, json.dumps(p)  # a bound pass ran
                assert got == datasets.oracle_run(ds, p), json.dumps(p)
    finally:
        capi.force_chain_variant(-1)


def test_plan_cache_replays_give_the_plain_results():
    """plan_cache: a plan seen twice becomes a prepared graph; replays, LRU
    eviction and table reloads all give the plain path's rows."""
    ds = datasets.dataset(0.05)
    pls = [plans.plan_star(2, 11), plans.plan_filter_sum(1994), plans.plan_date_join(1995),
           plans.plan_star(1, 3, 1993, 1996, 12)]
    with Engine(arena_bytes=1 << 30) as plain:
        load(plain, ds)
        want = [plain.execute(p).canonical() for p in pls]
    with Engine(arena_bytes=1 << 30, plan_cache=2) as eng:
        load(eng, ds)
        for _ in range(4):  # two plans fit the cache: the others keep being evicted and prepared again
            for p, w in zip(pls, want):
                assert eng.execute(p).canonical() == w
                assert eng.last_plan_ms() > 0
        # a reload into the same buffers with the same per-segment min/max
        # keeps the prepared plans, which read the new contents
        lo = ds["lineorder"]
        lo2 = {c: (a[::-1].copy() if c == 12 else a) for c, a in lo.items()}  # revenue permuted
        eng.load_table("lineorder", lo2)
        ds2 = dict(ds)
        ds2["lineorder"] = lo2
        for _ in range(3):
            assert eng.execute(pls[0]).canonical() == datasets.oracle_run(ds2, pls[0])
        # statistics that change (wider brand range: another group-by size)
        # drop them
        part3 = {c: (a + 1000 if c == 4 else a) for c, a in ds["part"].items()}
        eng.load_table("part", part3)
        ds3 = dict(ds2)
        ds3["part"] = part3
        for _ in range(3):
            assert eng.execute(pls[0]).canonical() == datasets.oracle_run(ds3, pls[0])


def test_order_by_on_the_device():
    """order_by: rows come out ordered by the plan's SORT collation (stable:
    ties keep row order), also across segments and on uint64 sums."""
    ds = datasets.dataset(0.05)
    star = plans.plan_star(2, 11)  # SORT on (d_year, p_brand1), ascending
    by_sum = json.loads(json.dumps(star))
    by_sum["rels"][-1]["collation"] = [{"field": 2, "direction": "DESCENDING", "nulls": "LAST"},
                                       {"field": 0, "direction": "ASCENDING", "nulls": "LAST"}]
    b = plans.PlanBuilder()  # a large, multi-segment result
    b.scan("lineorder")
    b.filter(plans.search(11, 2, 3))
    b.project([plans.col(5), plans.col(9)])
    b.sort([1, 0])
    wide = b.plan()
    wide["rels"][-1]["collation"][0]["direction"] = "DESCENDING"
    with Engine(arena_bytes=1 << 30, segment_rows=1 << 14) as plain:
        load(plain, ds)
        rows = {i: plain.execute(p).rows() for i, p in enumerate((star, by_sum, wide))}
    with Engine(arena_bytes=1 << 30, segment_rows=1 << 14, order_by=True, plan_cache=2) as eng:
        load(eng, ds)
        for _ in range(2):
            assert eng.execute(star).rows() == sorted(rows[0], key=lambda r: (r[0], r[1]))
            assert eng.execute(by_sum).rows() == sorted(rows[1], key=lambda r: (-r[2], r[0]))
            got = eng.execute(wide).rows()
            assert len(got) > 1 << 15  # rows from many 16K-row segments
            assert got == sorted(rows[2], key=lambda r: (-r[1], r[0]))


@pytest.mark.parametrize("fuse", [False, True])
def test_more_ssb_shapes_match_the_oracle(fuse):
    """Three group-by keys over three dimensions (SSB flight 3, with the
    region filter and with OR-of-two-points city filters) and the four-join
    profit shape (flight 4: revenue - supplycost, two semi joins)."""
    ds = datasets.dataset(0.05)
    cases = [plans.plan_customer_supplier_date(2), plans.plan_customer_supplier_date(0, 1992, 1993),
             plans.plan_customer_supplier_date(0, 1992, 1998, city_points=(21, 27)),
             plans.plan_profit(1), plans.plan_profit(3, (2, 4))]
    with Engine(arena_bytes=1 << 30, fuse=fuse, segment_rows=1 << 16) as eng:
        load(eng, ds)
        for plan in cases:
            got = eng.execute(plan).canonical()
            assert got == datasets.oracle_run(ds, plan, 1 << 16), json.dumps(plan)
            assert len(got) > 0


def test_wide_chains_split_only_when_order_does_not_matter():
    """An aggregating chain over more than four fact columns runs as two
    specialised passes when its flag-only ops can go first (the profit
    shape); with a fact filter whose ops combine with OR (order matters) it
    stays one pass.  Both give the oracle's rows, on every variant."""
    ds = datasets.dataset(0.05)
    b = plans.PlanBuilder()  # profit shape plus an OR fact filter in front
    f = b.scan("lineorder")
    f = b.filter(plans.OR(plans.expr("<", plans.col(8), plans.lit(20)), plans.search(11, 8, 10)))
    c = b.scan("customer")
    c = b.filter(plans.expr("==", plans.col(5), plans.lit(1)))
    j1 = b.join(f, c, 2, 17 + 0)
    s = b.scan("supplier")
    s = b.filter(plans.expr("==", plans.col(5), plans.lit(1)))
    j2 = b.join(j1, s, 4, 25 + 0, "semi")
    p = b.scan("part")
    p = b.filter(plans.search_points(2, 0, 1))
    j3 = b.join(j2, p, 3, 32 + 0, "semi")
    d = b.scan("ddate")
    b.join(j3, d, 5, 41 + 0)
    b.project([plans.col(41 + 4), plans.col(17 + 4), plans.expr("-", plans.col(12), plans.col(13))])
    b.aggregate([0, 1], 2)
    with_or = b.plan()
    cases = [plans.plan_profit(1), plans.plan_profit(2, (1, 3)), with_or]
    want = [datasets.oracle_run(ds, p) for p in cases]
    try:
        for variant in (-1, 0, 5, 7):
            capi.force_chain_variant(variant)
            with Engine(arena_bytes=1 << 30) as eng:
                load(eng, ds)
                for plan, w in zip(cases, want):
                    assert eng.execute(plan).canonical() == w, (variant, json.dumps(plan))
    finally:
        capi.force_chain_variant(-1)
    assert all(len(w) > 0 for w in want)


@pytest.mark.parametrize("fuse", [False, True])
def test_reljson_plans_give_the_idl_plans_rows(fuse):
    """SSB q1.1, q2.1 and q3.1 written in Calcite's RelJson dialect run on the
    device and give the rows of the same plans in the IDL shape, which are
    the oracle's."""
    from tests import test_reljson_cpu as R

    ds = datasets.dataset(0.05)
    idl = R.idl_plans()
    with Engine(arena_bytes=1 << 30, fuse=fuse, segment_rows=1 << 16) as eng:
        load(eng, ds)
        for name in ("q11", "q21", "q31"):
            want = datasets.oracle_run(ds, idl[name], 1 << 16)
            assert eng.execute(idl[name]).canonical() == want, name
            assert eng.execute(R.reljson(name)).canonical() == want, name
            assert len(want) > 0
