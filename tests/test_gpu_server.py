"""The served form on the GPU: plans arriving as a Poisson stream are admitted
against a device budget and batched while others run.  Every result must be
the one the plan gives alone (exactly: integer keys and uint64 sums), and the
plain one-at-a-time replay of the same trace must give the same results."""
import numpy as np
import pytest

from sycldb_gb300 import capi, plans, ssb, workloads
from sycldb_gb300.engine import Engine, Server, replay_plain
from tests import datasets, naive

pytestmark = pytest.mark.gpu

SF = 0.2


@pytest.fixture(scope="module")
def ds():
    return datasets.dataset(SF)


def make_engine(ds, **kw):
    eng = Engine(arena_bytes=1 << 30, **kw)
    for name, cols in ds.items():
        eng.load_table(name, cols)
    return eng


def trace(rate, n, seed=5):
    reqs = workloads.poisson_stream(rate, n, seed=seed)
    return [r.plan for r in reqs], [r.t for r in reqs]


@pytest.mark.parametrize("seg", [0, 1 << 18])
def test_each_result_is_the_same_alone_and_in_the_mix(ds, seg):
    pls, at = trace(2000, 240)
    with make_engine(ds, segment_rows=seg) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        with Server(eng, budget_bytes=8 << 30) as srv:
            st, lat, res, wall = srv.replay(pls, at)
            stats = srv.stats()
        assert st == [capi.SDB_OK] * len(pls)
        assert [r.canonical() for r in res] == alone
        assert all(x >= 0 for x in lat) and wall > 0
        assert stats["completed"] == len(pls) and stats["failed"] == 0
        assert stats["batches"] < len(pls)  # requests were batched
        assert stats["peak_device_bytes"] <= stats["budget_bytes"]
        pst, plat, pres, pwall = replay_plain(eng, pls, at)
        assert pst == [capi.SDB_OK] * len(pls)
        assert [r.canonical() for r in pres] == alone
    # a few against the oracle too
    for i in (0, 1, 2, 3, 57, 150):
        assert alone[i] == datasets.oracle_run(ds, pls[i], seg or None)


def test_submit_and_next_burst(ds):
    pls, _ = trace(1000, 60, seed=9)
    with make_engine(ds) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        with Server(eng, budget_bytes=4 << 30, slots=2, max_batch=16) as srv:
            ids = [srv.submit(p) for p in pls]
            got = {}
            for _ in pls:
                rid, st, res, ms, err = srv.next(timeout_ms=60_000)
                assert st == capi.SDB_OK, err
                got[rid] = res.canonical()
            stats = srv.stats()
            with pytest.raises(capi.SdbError) as e:
                srv.next(timeout_ms=10)
            assert e.value.status == capi.SDB_ERR_TIMEOUT
    assert [got[i] for i in ids] == alone
    assert 1 < stats["max_batch_plans"] <= 16


def test_admission_under_a_small_budget(ds):
    """A budget that holds only a few plans at once: everything still
    finishes, correctly, and in-flight memory never exceeds the budget; bad
    plans and plans larger than the whole budget fail alone."""
    pls, at = trace(3000, 80, seed=13)
    with make_engine(ds) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        budget = 24 << 20
        with Server(eng, budget_bytes=budget, slots=4) as srv:
            st, lat, res, wall = srv.replay(pls, at)
            stats = srv.stats()
            bad = srv.submit(plans.plan_filter_sum(1994, fact_tag=77))  # no such table
            rid, s_bad, r_bad, _, err = srv.next(timeout_ms=30_000)
        assert st == [capi.SDB_OK] * len(pls)
        assert [r.canonical() for r in res] == alone
        assert stats["peak_device_bytes"] <= budget
        assert rid == bad and s_bad == capi.SDB_ERR_INVALID and r_bad is None and "not found" in err
        with Server(eng, budget_bytes=1 << 20) as tiny:
            rid = tiny.submit(pls[0])
            _, s, r, _, err = tiny.next(timeout_ms=30_000)
        assert s == capi.SDB_ERR_NOMEM and r is None


def test_server_is_reusable_after_destroy(ds):
    pls, at = trace(500, 20, seed=21)
    with make_engine(ds) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        for _ in range(2):
            with Server(eng, budget_bytes=2 << 30) as srv:
                st, _, res, _ = srv.replay(pls, at)
            assert [r.canonical() for r in res] == alone
        assert eng.execute(pls[0]).canonical() == alone[0]  # the engine works again afterwards


def test_large_chains_run_on_their_own_in_the_mix():
    """A 9 M-row fact table: its aggregating chains are above the batch's
    single-launch size (2^23 rows), so the server's batches launch them with
    the single-chain kernel between the build launch and the chain batch.
    Results stay those of each plan alone."""
    big = datasets.dataset(1.5, fact_cols=(3, 4, 5, 8, 9, 11, 12))
    assert big["lineorder"][5].size >= 1 << 23
    pls, at = trace(3000, 48, seed=9)
    with make_engine(big) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        with Server(eng, budget_bytes=8 << 30) as srv:
            st, lat, res, wall = srv.replay(pls, at)
            stats = srv.stats()
        assert st == [capi.SDB_OK] * len(pls)
        assert [r.canonical() for r in res] == alone
        assert stats["batches"] < len(pls)
        with eng.batch(pls[:12]) as b:
            assert [r.canonical() for r in b.run()] == alone[:12]
            assert b.stats()["batched_chains"] == 0  # every fact chain is large
            # twelve plans of four kinds over one table: some share a scan
            assert b.stats()["paired_chains"] >= 2


def _naive_of(kind, plan, fact, dims):
    """The naive evaluator's rows for a served request, from its plan's
    constants (the plan builders of sycldb_gb300.plans)."""
    rels = plan["rels"]
    if kind == "filter_sum":
        cond = rels[1]["condition"]["operands"]
        lo = int(cond[0]["operands"][1]["literal"]["rangeSet"][0][1])
        d_lo = int(cond[1]["operands"][1]["literal"]["rangeSet"][0][1])
        d_hi = int(cond[1]["operands"][1]["literal"]["rangeSet"][0][2])
        q = int(cond[2]["operands"][1]["literal"]["value"])
        return naive.filter_sum_vec(fact, lo // 10000, d_lo, d_hi, q)
    if kind == "date_join":
        rs = rels[1]["condition"]["operands"][1]["literal"]["rangeSet"][0]
        y0 = int(rels[3]["condition"]["operands"][1]["literal"]["rangeSet"][0][1])
        return naive.date_join_vec(fact, dims["ddate"], y0, int(rs[1]), int(rs[2]))
    region = int(rels[2]["condition"]["operands"][1]["literal"]["value"])
    pf = rels[5]["condition"]
    if kind == "star":
        return naive.star_vec(fact, dims["supplier"], dims["part"], dims["ddate"], region,
                              int(pf["operands"][1]["literal"]["value"]))
    cat = int(pf["operands"][0]["operands"][1]["literal"]["value"])
    b = pf["operands"][1]["operands"][1]["literal"]["rangeSet"][0]
    y = rels[8]["condition"]["operands"][1]["literal"]["rangeSet"][0]
    return naive.star_vec(fact, dims["supplier"], dims["part"], dims["ddate"], region, cat, int(y[1]), int(y[2]),
                          int(b[2]) - int(b[1]) + 1)


def test_served_sf50_every_plan_kind_matches_naive():
    """The served configuration's table at full size: SF50, 300 M fact rows
    in two 2^28-row segments, SF50 dimensions.  A Poisson stream with every
    plan kind goes through the server and the plain path; two requests of
    each kind are checked against the independent naive evaluator."""
    import torch

    sf = 50.0
    n = ssb.fact_rows(sf)
    cols = (3, 4, 5, 8, 9, 11, 12)
    dims = ssb.gen_dims(sf)
    reqs = workloads.poisson_stream(1000.0, 32, seed=ssb.SEED + 5)
    kinds = {}
    for i, r in enumerate(reqs):
        kinds.setdefault(r.kind, []).append(i)
    assert set(kinds) == {"filter_sum", "date_join", "star", "batch_star"}
    pls, at = [r.plan for r in reqs], [r.t for r in reqs]
    fact = ssb.gen_lineorder_device(n, cols, sf)
    with Engine() as eng:
        eng.load_table("lineorder", fact)
        for t in ("supplier", "part", "ddate"):
            eng.load_table(t, dims[t])
        pst, _, pres, _ = replay_plain(eng, pls, at)
        with Server(eng, budget_bytes=60 << 30) as srv:
            sst, _, sres, _ = srv.replay(pls, at)
    del fact
    torch.cuda.empty_cache()
    assert pst == [capi.SDB_OK] * len(pls) and sst == [capi.SDB_OK] * len(pls)
    plain = [r.canonical() for r in pres]
    assert [r.canonical() for r in sres] == plain
    host = ssb.gen_lineorder_host(n, cols, sf)
    for kind, idx in kinds.items():
        for i in idx[:2]:
            want = _naive_of(kind, pls[i], host, dims)
            assert plain[i] == want, (kind, i)
            assert len(want) > 0


@pytest.mark.parametrize("direct", [True, False])
def test_lone_requests_at_an_idle_server_run_directly(ds, direct):
    """At a low arrival rate most requests find the server idle: they run at
    once through the plain path (no sizing pass, no batch); with direct off,
    every one goes through a batch.  Results are each plan's own either way."""
    pls, at = trace(50, 40, seed=31)
    with make_engine(ds) as eng:
        alone = [eng.execute(p).canonical() for p in pls]
        with Server(eng, budget_bytes=8 << 30, direct=direct) as srv:
            st, lat, res, wall = srv.replay(pls, at)
            stats = srv.stats()
        assert st == [capi.SDB_OK] * len(pls)
        assert [r.canonical() for r in res] == alone
        if direct:
            assert stats["direct_plans"] > len(pls) // 2
            assert stats["direct_plans"] + stats["batched_plans"] == len(pls)
        else:
            assert stats["direct_plans"] == 0 and stats["batched_plans"] == len(pls)
        # a budget below the engine's own memory turns the direct path off
        with Server(eng, budget_bytes=256 << 20) as small:
            st2, _, res2, _ = small.replay(pls[:8], at[:8])
            assert small.stats()["direct_plans"] == 0
        assert [r.canonical() for r in res2] == alone[:8]
