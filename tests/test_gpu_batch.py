"""The batched form on the GPU: many plans prepared once and run together
(one CUDA graph; the plans' aggregating fused chains in one persistent launch
per chain shape) must give, plan by plan, exactly the rows each plan gives
alone, and those must match the oracle."""
import numpy as np
import pytest

from sycldb_gb300 import capi, plans, ssb, workloads
from sycldb_gb300.engine import Engine
from tests import datasets, naive

pytestmark = pytest.mark.gpu

# fact partitions of uneven size, tile edges included (a tile is 1024 rows)
SIZES = [1, 1000, 1023, 1024, 1025, 4097, 65_536, 300_001, 1_234_567]
DIM_SF = 0.2
FACT_COLS = (3, 4, 5, 8, 9, 11, 12)


def small_tables():
    dims = ssb.gen_dims(DIM_SF)
    tables = {n: dims[n] for n in ("supplier", "part", "ddate")}
    for p, n in enumerate(SIZES):
        tables["lineorder@%d" % p] = ssb.gen_lineorder_host(n, FACT_COLS, DIM_SF, salt=p + 1)
    return tables


def small_plans():
    rng = np.random.default_rng(11)
    out = []
    for p in range(len(SIZES)):
        out.append(workloads.draw_star_params(rng).plan(fact_tag=p))
    out.append(plans.plan_star(1, 3, fact_tag=8))                 # the full star shape, no year/brand filter
    out.append(plans.plan_filter_sum(1994, 1, 3, 25, fact_tag=7))  # SUM terminal: another chain shape
    out.append(plans.plan_date_join(1995, fact_tag=6))             # range + join + projection shape
    out.append(plans.plan_filter_sum(1996, 4, 6, 30, fact_tag=0))  # a one-row partition
    out.append(plans.plan_star(2, 11, 1993, 1997, 40, fact_tag=5))
    out.append(plans.plan_star(2, 11, 1993, 1997, 40, fact_tag=5))  # the same plan twice
    return out


@pytest.fixture(scope="module")
def tables():
    return small_tables()


@pytest.fixture(scope="module")
def oracle_rows(tables):
    return [datasets.oracle_run(tables, pl) for pl in small_plans()]


def make_engine(tables, **kw):
    eng = Engine(arena_bytes=1 << 30, **kw)
    for name, cols in tables.items():
        eng.load_table(name, cols)
    return eng


@pytest.mark.parametrize("eager", [False, True])
@pytest.mark.parametrize("chain_batch", [True, "builds", False])
def test_batch_equals_each_plan_alone_and_the_oracle(tables, oracle_rows, eager, chain_batch):
    pls = small_plans()
    with make_engine(tables) as eng:
        alone = [eng.execute(pl).canonical() for pl in pls]
        assert alone == oracle_rows
        with eng.batch(pls, eager=eager, chain_batch=chain_batch) as b:
            for _ in range(3):  # replays re-zero the batch's tables
                got = [r.canonical() for r in b.run()]
                assert got == alone
            st = b.stats()
        assert st["n_plans"] == len(pls)
        assert st["graph"] == (0 if eager else 1)
        assert st["kernels_per_run"] > 0
        if chain_batch is True:
            assert st["batched_chains"] == len(pls)  # every plan ends in an aggregating chain
            assert st["batched_builds"] > 0          # dimension filters + builds in one launch
            assert st["chain_launches"] == 4         # star, filter-sum and date-join shapes; the builds
        elif chain_batch == "builds":
            assert st["batched_chains"] == 0 and st["batched_builds"] > 0 and st["chain_launches"] == 1
        else:
            assert st["batched_chains"] == 0 and st["batched_builds"] == 0


def test_batch_with_several_segments_per_plan(tables, oracle_rows):
    """4096-row segments: one chain per segment and plan, all in the batch."""
    pls = small_plans()
    with make_engine(tables, segment_rows=4096) as eng:
        with eng.batch(pls) as b:
            got = [r.canonical() for r in b.run()]
            assert b.stats()["batched_chains"] > len(pls)
    assert got == oracle_rows


def test_batch_operator_at_a_time_engine(tables, oracle_rows):
    """Without fusion nothing goes to a chain batch; the graph still runs
    every plan."""
    pls = small_plans()
    with make_engine(tables, fuse=False) as eng:
        with eng.batch(pls) as b:
            got = [r.canonical() for r in b.run()]
            assert b.stats()["batched_chains"] == 0
    assert got == oracle_rows


def test_batches_and_plain_executes_interleave(tables, oracle_rows):
    pls = small_plans()
    with make_engine(tables) as eng:
        b1 = eng.batch(pls[:6])
        b2 = eng.batch(pls[6:])
        for _ in range(2):
            r1 = [r.canonical() for r in b1.run()]
            single = eng.execute(pls[3]).canonical()
            r2 = [r.canonical() for r in b2.run()]
            assert r1 == oracle_rows[:6]
            assert r2 == oracle_rows[6:]
            assert single == oracle_rows[3]
        b1.close()
        b2.close()


def test_batch_run_without_unpacking_and_errors(tables, oracle_rows):
    pls = small_plans()
    with make_engine(tables) as eng:
        with eng.batch(pls[:3]) as b:
            assert b.run(unpack=False) is None
            assert [r.canonical() for r in b.run()] == oracle_rows[:3]
        bad = plans.plan_filter_sum(1994, fact_tag=99)  # no such table
        with pytest.raises(capi.SdbError) as e:
            eng.batch([pls[0], bad])
        assert e.value.status == capi.SDB_ERR_INVALID
        assert "not found" in str(e.value)
        assert eng.execute(pls[0]).canonical() == oracle_rows[0]  # engine still usable


def test_batched_form_full_size_equals_plain():
    """64 star-join plans over fact partitions of 1M..50M rows (lognormal),
    SF20 dimensions: the batch gives each plan's own result, and every plan's
    rows are those of the independent naive evaluator over its partition
    (with the plan's region, category, year and brand windows)."""
    wl = workloads.batch_workload()
    dims = ssb.gen_dims(wl.dim_sf, wl.seed)
    with Engine() as eng:
        workloads.load_batch_tables(eng, wl, device=True, dims=dims)
        pls = wl.plans()
        alone = [eng.execute(pl).canonical() for pl in pls]
        with eng.batch(pls) as b:
            got = [r.canonical() for r in b.run()]
            st = b.stats()
    assert got == alone
    for p, (n, prm) in enumerate(zip(wl.rows, wl.params)):
        fact = ssb.gen_lineorder_host(n, workloads.STAR_COLS, wl.dim_sf, wl.seed, salt=p + 1)
        want = naive.star_vec(fact, dims["supplier"], dims["part"], dims["ddate"], prm.region, prm.category,
                              prm.year_lo, prm.year_hi, prm.brand_count)
        assert alone[p] == want, p
    # the fact chains of partitions under 2^23 rows in one launch (larger ones
    # run the single-chain kernel on their own), the 192 dimension builds in one
    small = sum(1 for r in wl.rows if r < (1 << 23))
    assert 0 < small < 64
    assert st["batched_chains"] == small and st["batched_builds"] == 192 and st["chain_launches"] == 2
    groups = [len(r) for r in alone]
    assert max(groups) <= 280 and all(g <= p.max_groups for g, p in zip(groups, wl.params))


@pytest.mark.parametrize("variant", [3, 4, 5, 6, 7, 8])
def test_batch_under_each_specialised_variant(tables, oracle_rows, variant):
    """The chain batch with every shape-specialised variant (dense, compacted
    with a 3- or 2-stage ring, rows carried across tiles)."""
    pls = small_plans()
    try:
        capi.force_chain_variant(variant)
        with make_engine(tables) as eng:
            with eng.batch(pls) as b:
                got = [r.canonical() for r in b.run()]
                assert b.stats()["chain_launches"] == 4
            alone = [eng.execute(pl).canonical() for pl in pls]
    finally:
        capi.force_chain_variant(-1)
    assert got == oracle_rows
    assert alone == oracle_rows


@pytest.mark.parametrize("chain_batch", [True, "builds", False])
def test_batch_with_split_and_three_key_chains(chain_batch):
    """Flight-4 plans (their chains split in two passes: the flags pass runs
    before the chain batch) and flight-3 plans (three full probes, three
    keys) in one batch: each plan's rows as alone."""
    ds = datasets.dataset(0.05)
    pls = [plans.plan_profit(1), plans.plan_customer_supplier_date(2), plans.plan_profit(3, (2, 4)),
           plans.plan_customer_supplier_date(0, 1992, 1993), plans.plan_star(1, 3)]
    with Engine(arena_bytes=1 << 30) as eng:
        for name, cols in ds.items():
            eng.load_table(name, cols)
        alone = [eng.execute(p).canonical() for p in pls]
        with eng.batch(pls, chain_batch=chain_batch) as b:
            for _ in range(2):
                assert [r.canonical() for r in b.run()] == alone
    assert alone[0] == datasets.oracle_run(ds, pls[0])
    assert all(len(a) > 0 for a in alone)


@pytest.mark.parametrize("segment_rows", [0, 1 << 20])
def test_shared_scans_pair_plans_over_the_same_rows(tables, segment_rows):
    """Star, date-join and filter-project-sum plans over one fact table, each
    with its own literals: a batch runs two chains of one shape over the
    same rows as one paired pass (each tile staged once), and every plan's
    rows equal its rows alone, the batch's without shared scans and the
    oracle's.  With several segments per plan, chains pair segment by
    segment."""
    pls = [plans.plan_star(1, 3, fact_tag=8), plans.plan_star(2, 11, fact_tag=8), plans.plan_star(3, 20, fact_tag=8),
           plans.plan_date_join(1995, fact_tag=8), plans.plan_date_join(1997, fact_tag=8),
           plans.plan_filter_sum(1994, 1, 3, 25, fact_tag=8), plans.plan_filter_sum(1993, 4, 6, 35, fact_tag=8)]
    try:
        capi.force_chain_variant(8)  # the variant that pairs, at every size
        with make_engine(tables, segment_rows=segment_rows) as eng, \
                make_engine(tables, segment_rows=segment_rows, shared_scans=False) as apart:
            alone = [eng.execute(pl).canonical() for pl in pls]
            assert alone[0] == datasets.oracle_run(tables, pls[0])
            assert alone[3] == datasets.oracle_run(tables, pls[3])
            assert alone[5] == datasets.oracle_run(tables, pls[5])
            paired = {}
            for name, e in (("shared", eng), ("apart", apart)):
                for eager in (False, True):
                    with e.batch(pls, eager=eager, chain_batch="builds") as b:
                        for _ in range(2):  # replays re-zero the group tables
                            assert [r.canonical() for r in b.run()] == alone
                        paired[name, eager] = b.stats()["paired_chains"]
    finally:
        capi.force_chain_variant(-1)
    # a pair of stars (the third alone), of date joins and of filter-sums
    # (per segment, where a plan's segment chains lead its work)
    for eager in (False, True):
        assert paired["apart", eager] == 0
        assert paired["shared", eager] == 6 if segment_rows == 0 else paired["shared", eager] in (6, 12)


@pytest.mark.parametrize("part", [0, 1, 4, 5, 6])
def test_shared_scans_at_tile_edges(tables, part):
    """The paired pass on fact partitions of 1, 1000, 1025, 4097 and 65,536
    rows (below one tile, around tile edges): two star plans and two
    filter-project-sum plans share scans, each plan's rows equal its rows
    alone and, for the first of each shape, the oracle's."""
    pls = [plans.plan_star(1, 3, fact_tag=part), plans.plan_star(2, 11, fact_tag=part),
           plans.plan_filter_sum(1994, 1, 3, 25, fact_tag=part), plans.plan_filter_sum(1993, 4, 6, 35, fact_tag=part)]
    try:
        capi.force_chain_variant(8)  # the variant that pairs, at every size
        with make_engine(tables) as eng:
            alone = [eng.execute(pl).canonical() for pl in pls]
            assert alone[0] == datasets.oracle_run(tables, pls[0])
            assert alone[2] == datasets.oracle_run(tables, pls[2])
            with eng.batch(pls, chain_batch="builds") as b:
                for _ in range(2):
                    assert [r.canonical() for r in b.run()] == alone
                assert b.stats()["paired_chains"] == 4
    finally:
        capi.force_chain_variant(-1)
