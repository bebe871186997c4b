"""The two SF1 configurations at their stated size (6,000,000 fact rows) on
the GPU, against the oracle and the independent naive evaluator:

* filter-project-aggregate: orderdate within one calendar year, discount in
  [1, 3], quantity < 25; SUM(extendedprice * discount) into one uint64;
* filter + date join + group-by: discount in [4, 6], date dimension filtered
  on a two-year range; group by year, SUM(extendedprice * discount).

Each runs fused, operator at a time, in two segments, and through the
prepared-plan path (plan cache), and every form must give the oracle's rows
(executor/ddor_executor.cpp:105-216; kernels/aggregation.hpp:208-228,278-344;
kernels/join.hpp:256-312)."""
import pytest

from sycldb_gb300 import plans, ssb
from sycldb_gb300.engine import Engine
from tests import datasets, naive

pytestmark = pytest.mark.gpu

SF = 1.0
FACT_COLS = (5, 8, 9, 11)


@pytest.fixture(scope="module")
def ds():
    return datasets.dataset(SF, fact_cols=FACT_COLS)


def _engine(ds, **kw):
    eng = Engine(arena_bytes=2 << 30, **kw)
    eng.load_table("lineorder", ds["lineorder"])
    eng.load_table("ddate", ds["ddate"])
    return eng


CASES = [("filter_sum", 1992), ("filter_sum", 1994), ("filter_sum", 1998),
         ("date_join", 1992), ("date_join", 1994), ("date_join", 1997)]


def _plan(kind, year):
    return plans.plan_filter_sum(year) if kind == "filter_sum" else plans.plan_date_join(year)


def _naive(ds, kind, year):
    f = ds["lineorder"]
    if kind == "filter_sum":
        return naive.filter_sum_vec(f, year)
    return naive.date_join_vec(f, ds["ddate"], year)


@pytest.mark.parametrize("kind,year", CASES)
def test_sf1_configuration_matches_oracle_and_naive(ds, kind, year):
    assert ds["lineorder"][5].size == ssb.fact_rows(SF) == 6_000_000
    plan = _plan(kind, year)
    want = datasets.oracle_run(ds, plan)
    assert want == _naive(ds, kind, year)
    assert len(want) == (1 if kind == "filter_sum" else 2)
    for kw in ({"fuse": True}, {"fuse": False}, {"fuse": True, "segment_rows": 1 << 22},
               {"fuse": False, "segment_rows": 1 << 22}):
        with _engine(ds, **kw) as eng:
            assert eng.execute(plan).canonical() == want, kw
    with _engine(ds, fuse=True, plan_cache=2) as eng:  # prepared plan replays
        for _ in range(3):
            assert eng.execute(plan).canonical() == want


@pytest.mark.parametrize("variant", [0, 3, 4, 5, 6, 7, 8])
def test_sf1_configurations_on_every_fused_variant(ds, variant):
    from sycldb_gb300 import capi

    want = {c: datasets.oracle_run(ds, _plan(*c)) for c in CASES[:2] + CASES[3:5]}
    try:
        capi.force_chain_variant(variant)
        with _engine(ds, fuse=True) as eng:
            for c, w in want.items():
                assert eng.execute(_plan(*c)).canonical() == w, (variant, c)
    finally:
        capi.force_chain_variant(-1)
