"""The oracle's executor layer pinned to the reference's own executor: the
same plans over the same seeded tables through SYCLDB's execute_ddor_plan
(models/transient_table.hpp, executor/ddor_executor.cpp,
operations/preprocessing.cpp; compiled from the reference checkout against
host shims by oracle/build_oracle.py) and through the oracle's restatement
(oracle/oracle.py), with 2^28-row segments and with 4096-row segments (the
phase and segment-merge logic over many segments).  The golden rows the GPU
tests compare the engine with are checked against the reference executor
too.  Skipped where the checkout is absent (the library is not built)."""
import json
import os

import pytest

from oracle import ref_exec
from sycldb_gb300 import plans as P
from tests import datasets

pytestmark = pytest.mark.skipif(not (ref_exec.available(0) and ref_exec.available(4096)),
                                reason="reference executor checker not built (no reference checkout)")

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN = json.load(open(os.path.join(HERE, "plans.json")))


@pytest.mark.parametrize("seg", [0, 4096])
@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_golden_rows_are_the_reference_executors(case, seg):
    ds = datasets.dataset(case["sf"], case["seed"])
    assert [list(r) for r in ref_exec.run(ds, case["plan"], seg)] == case["rows"]


def _shapes():
    """The benchmark and widened shapes, and plans that exercise the
    executor's quirks: OR under AND (the parent operator handed to the first
    child), SEARCH points and reversed ranges, column-column comparisons,
    literal projections, every binary operator, a plan ending in a filter."""
    out = [P.plan_star(2, 11), P.plan_star(1, 3, 1993, 1996, 12), P.plan_date_join(1995), P.plan_filter_sum(1996),
           P.plan_customer_supplier_date(2), P.plan_customer_supplier_date(0, 1992, 1993),
           P.plan_customer_supplier_date(0, 1992, 1998, city_points=(21, 27)), P.plan_profit(1), P.plan_profit(3, (2, 4))]
    b = P.PlanBuilder()
    b.scan("lineorder")
    b.filter(P.AND(P.expr("<=", P.col(8), P.lit(30)),
                   P.OR(P.search_points(11, 2, 7), P.expr(">", P.col(9), P.col(12)))))
    b.project([P.expr("-", P.col(9), P.col(13)), P.lit(3)])
    b.aggregate([], 0)
    out.append(b.plan())
    for op in ["*", "/", "+", "-"]:
        b = P.PlanBuilder()
        b.scan("lineorder")
        b.filter(P.expr("<>", P.col(11), P.lit(0)))
        b.project([P.col(8), P.expr(op, P.col(9), P.col(11)), P.expr(op, P.lit(1000), P.col(11))])
        b.aggregate([0], 1)
        out.append(b.plan())
    b = P.PlanBuilder()
    b.scan("lineorder")
    b.filter(P.AND(P.search(5, 19941231, 19940101), P.search(11, 1, 3), P.expr("<", P.col(8), P.lit(25))))
    b.project([P.expr("*", P.col(9), P.col(11))])
    b.aggregate([], 0)
    out.append(b.plan())
    b = P.PlanBuilder()  # ends in a filter (no aggregate)
    b.scan("lineorder")
    b.filter(P.AND(P.expr("==", P.col(11), P.lit(10)), P.expr("<", P.col(8), P.lit(3))))
    b.project([P.col(5), P.col(9)])
    out.append(b.plan())
    return out


@pytest.mark.parametrize("seg", [0, 4096])
def test_oracle_executor_matches_the_reference_executor(seg):
    ds = datasets.dataset(0.02)
    for plan in _shapes():
        want = ref_exec.run(ds, plan, seg)
        got = datasets.oracle_run(ds, plan, seg or None)
        assert [tuple(r) for r in got] == want, json.dumps(plan)
