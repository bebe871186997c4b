"""The oracle's executor restatement against the independent naive evaluator,
plus the executor quirks the reference has (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O
from sycldb_gb300 import plans
from tests import datasets, naive


@pytest.mark.parametrize("year", [1992, 1993, 1997])
@pytest.mark.parametrize("seg", [None, 4096])
def test_filter_sum(year, seg):
    ds = datasets.dataset(0.01)
    got = datasets.oracle_run(ds, plans.plan_filter_sum(year), seg)
    assert got == naive.filter_sum(ds["lineorder"], year)


@pytest.mark.parametrize("year0", [1992, 1995, 1997])
@pytest.mark.parametrize("seg", [None, 8192])
def test_date_join(year0, seg):
    ds = datasets.dataset(0.01)
    got = datasets.oracle_run(ds, plans.plan_date_join(year0), seg)
    assert got == naive.date_join(ds["lineorder"], ds["ddate"], year0)
    assert len(got) == 2


@pytest.mark.parametrize("region,category", [(0, 0), (1, 1), (4, 24), (2, 13)])
@pytest.mark.parametrize("seg", [None, 16384])
def test_star(region, category, seg):
    ds = datasets.dataset(0.05)
    got = datasets.oracle_run(ds, plans.plan_star(region, category), seg)
    want = naive.star(ds["lineorder"], ds["supplier"], ds["part"], ds["ddate"], region, category)
    assert got == want
    assert len(got) > 0


@pytest.mark.parametrize("args", [(3, 7, 1993, 1995, 5), (0, 2, 1998, 1998, 1), (1, 20, 1992, 1998, 40)])
def test_star_batched_shape(args):
    r, c, ylo, yhi, nb = args
    ds = datasets.dataset(0.05)
    got = datasets.oracle_run(ds, plans.plan_star(r, c, ylo, yhi, nb))
    want = naive.star(ds["lineorder"], ds["supplier"], ds["part"], ds["ddate"], r, c, ylo, yhi, nb)
    assert got == want


def test_dag_order_defers_lineorder():
    """operations/preprocessing.cpp:60-66: the lineorder scan goes last among
    the sources."""
    p = plans.plan_star(1, 1)
    order = O.dag_topological_sort(p["rels"])
    assert order[:3] == [1, 4, 7]
    assert order.index(0) > order.index(5)


def test_group_by_discovery():
    p = plans.plan_star(1, 1)
    loaded, group_by, _ = O.parse_execution_info(p["rels"])
    assert group_by == {"ddate": 4, "part": 4}
    assert loaded["lineorder"] == {3, 4, 5, 12}
    assert loaded["supplier"] == {0, 5}


def _tiny_tables():
    fact = {c: np.zeros(8, np.int32) for c in range(17)}
    fact[8] = np.array([1, 2, 3, 4, 5, 6, 7, 8], np.int32)
    fact[9] = np.array([10, 20, 30, 40, 50, 60, 70, 80], np.int32)
    return {"lineorder": O.make_table("lineorder", fact)}


def test_parent_op_quirk():
    """A logical node passes ITS PARENT's op to its first child
    (models/transient_table.hpp:847-848): AND(x, OR(a, b)) computes
    (x AND a) OR b, not x AND (a OR b)."""
    b = plans.PlanBuilder()
    b.scan("lineorder")
    b.filter(plans.AND(plans.expr("<=", plans.col(8), plans.lit(4)),
                       plans.OR(plans.expr(">=", plans.col(8), plans.lit(3)),
                                plans.expr("==", plans.col(8), plans.lit(8)))))
    b.project([plans.col(9)])
    b.aggregate([], 0)
    ex = O.OracleExecutor(_tiny_tables())
    (s,) = ex.execute(b.plan())
    # (q <= 4 AND q >= 3) OR q == 8 -> q in {3, 4, 8} -> 30 + 40 + 80
    assert int(s[0]) == 150


def test_search_points_and_negative_sum():
    b = plans.PlanBuilder()
    b.scan("lineorder")
    b.filter(plans.search_points(8, 2, 7))
    b.project([plans.expr("-", plans.lit(0), plans.col(9))])
    b.aggregate([], 0)
    (s,) = O.OracleExecutor(_tiny_tables()).execute(b.plan())
    assert int(s[0]) == (-(20 + 70)) & 0xFFFFFFFFFFFFFFFF


def test_group_by_emits_zero_sum_slots():
    """A slot that received rows is emitted even when its sum is 0."""
    fact = {c: np.zeros(6, np.int32) for c in range(17)}
    fact[8] = np.array([1, 1, 2, 2, 3, 3], np.int32)
    fact[9] = np.array([5, -5, 0, 0, 7, 1], np.int32)
    t = {"lineorder": O.make_table("lineorder", fact)}
    b = plans.PlanBuilder()
    b.scan("lineorder")
    b.project([plans.col(8), plans.col(9)])
    b.aggregate([0], 1)
    got = O.canonical_rows(O.OracleExecutor(t).execute(b.plan()))
    assert got == [(1, 0), (2, 0), (3, 8)]
