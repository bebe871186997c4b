"""Plan ingestion in Calcite's RelJson dialect (the JSON the reference's
planner emits and SycldbJsonConverter turns into the Thrift IDL structs,
server/src/main/java/com/eurecom/calcite/SycldbJsonConverter.java:31-163):
hand-made RelJson plans of SSB q1.1, q2.1 and q3.1 parse into exactly the
IDL-shaped plans built independently with sycldb_gb300.plans, take the same
execution order, and the oracle's rows on them are the naive evaluator's."""
import ctypes
import json
import os

import pytest

from sycldb_gb300 import capi, plans
from tests import datasets, naive

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reljson")


def reljson(name: str) -> str:
    with open(os.path.join(HERE, name + ".json")) as f:
        return f.read()


def idl_plans():
    P = plans
    b = P.PlanBuilder()
    b.scan("lineorder")
    b.filter(P.AND(P.search(5, 19930101, 19940101), P.search(11, 1, 3), P.expr("<", P.col(8), P.lit(25))))
    b.project([P.expr("*", P.col(9), P.col(11))])
    b.aggregate([], 0)
    q11 = b.plan()

    b = P.PlanBuilder()
    f = b.scan("lineorder")
    p = b.scan("part")
    p = b.filter(P.expr("==", P.col(3), P.lit(1)))
    j = b.join(f, p, 3, 17)
    s = b.scan("supplier")
    s = b.filter(P.expr("==", P.col(5), P.lit(1)))
    j = b.join(j, s, 4, 26, "semi")
    d = b.scan("ddate")
    b.join(j, d, 5, 33)
    b.project([P.col(37), P.col(21), P.col(12)])
    b.aggregate([0, 1], 2)
    b.sort([0, 1])
    q21 = b.plan()

    b = P.PlanBuilder()
    f = b.scan("lineorder")
    c = b.scan("customer")
    c = b.filter(P.expr("==", P.col(5), P.lit(2)))
    j = b.join(f, c, 2, 17)
    s = b.scan("supplier")
    s = b.filter(P.expr("==", P.col(5), P.lit(2)))
    j = b.join(j, s, 4, 25)
    d = b.scan("ddate")
    d = b.filter(P.search(4, 1992, 1997))
    b.join(j, d, 5, 32)
    b.project([P.col(21), P.col(29), P.col(36), P.col(12)])
    b.aggregate([0, 1, 2], 3)
    b.sort([2, 3])
    q31 = b.plan()
    q31["rels"][-1]["collation"][1]["direction"] = "DESCENDING"
    return {"q11": q11, "q21": q21, "q31": q31}


# The operator spellings differ between the dialects ("=" in Calcite, "=="
# in the IDL plans of plans.py); the executor decodes both to EQ
# (kernels/selection.hpp:23-39 maps unknown strings to EQ as well).
_OP_ALIASES = {"=": "=="}


def semantic(plan: dict) -> dict:
    """What the executor uses of a parsed plan: names, field labels and
    types dropped, operator aliases unified."""
    def expr(e):
        out = {"exprType": e["exprType"]}
        if e["exprType"] == "COLUMN":
            out["input"] = e["input"]
        elif e["exprType"] == "EXPR":
            out["op"] = _OP_ALIASES.get(e["op"], e["op"])
            out["operands"] = [expr(o) for o in e["operands"]]
        else:
            out["literal"] = e["literal"]
        return out

    rels = []
    for r in plan["rels"]:
        q = {k: v for k, v in r.items() if k not in ("fields",)}
        if "condition" in q:
            q["condition"] = expr(q["condition"])
        if "exprs" in q:
            q["exprs"] = [expr(e) for e in q["exprs"]]
        if "aggs" in q:
            q["aggs"] = [{"agg": a["agg"], "operands": a["operands"], "distinct": a["distinct"]} for a in q["aggs"]]
        rels.append(q)
    return {"rels": rels}


@pytest.mark.parametrize("name", ["q11", "q21", "q31"])
def test_reljson_parses_to_the_idl_plan(name):
    got = capi.plan_to_idl(reljson(name))
    want = capi.plan_to_idl(idl_plans()[name])
    assert semantic(got) == semantic(want)
    assert [r["relOp"] for r in got["rels"]][0] == "TABLE_SCAN"


@pytest.mark.parametrize("name", ["q11", "q21", "q31"])
def test_reljson_takes_the_idl_plans_execution_order(name):
    L = capi.lib()
    orders = []
    for text in (reljson(name), json.dumps(idl_plans()[name])):
        n = ctypes.c_int()
        order = (ctypes.c_int * 64)()
        capi.check(L.sdb_plan_check(text.encode(), ctypes.byref(n), order, 64))
        orders.append(list(order[:n.value]))
    assert orders[0] == orders[1]


def test_idl_writer_round_trips():
    for p in list(idl_plans().values()) + [plans.plan_star(2, 11, 1993, 1996, 12), plans.plan_profit(1)]:
        once = capi.plan_to_idl(p)
        assert capi.plan_to_idl(once) == once


def test_oracle_rows_on_the_idl_plans_are_the_naive_rows():
    ds = datasets.dataset(0.05)
    q = idl_plans()
    f = ds["lineorder"]
    rows11 = datasets.oracle_run(ds, q["q11"])
    d, c, qty, p = f[5], f[11], f[8], f[9]
    import numpy as np

    m = (d >= 19930101) & (d <= 19940101) & (c >= 1) & (c <= 3) & (qty < 25)
    assert rows11 == [(int((p[m].astype(np.int64) * c[m]).sum()) & (2 ** 64 - 1),)]
    rows21 = datasets.oracle_run(ds, q["q21"])
    assert rows21 == naive.star_vec(f, ds["supplier"], ds["part"], ds["ddate"], 1, 1)
    assert len(datasets.oracle_run(ds, q["q31"])) > 0


@pytest.mark.parametrize("bad", [
    {"rels": [{"id": "0", "relOp": "com.eurecom.calcite.SycldbWindow", "table": ["ssb", "lineorder"]}]},
    {"rels": [{"id": "x0", "relOp": "com.eurecom.calcite.SycldbTableScan", "table": ["ssb", "lineorder"]}]},
    {"rels": [{"id": "0", "relOp": "com.eurecom.calcite.SycldbTableScan", "table": ["ssb", "lineorder"],
               "inputs": []},
              {"id": "1", "relOp": "com.eurecom.calcite.SycldbFilter",
               "condition": {"op": {"name": "="}, "operands": [{"input": 5}, {"literal": None}]}}]},
    {"rels": [{"id": "0", "relOp": "com.eurecom.calcite.SycldbTableScan", "table": ["ssb", "lineorder"],
               "inputs": []},
              {"id": "1", "relOp": "com.eurecom.calcite.SycldbFilter",
               "condition": {"op": {"kind": "EQUALS"}, "operands": [{"input": 5}, {"literal": 3}]}}]},
    {"rels": [{"id": "0", "relOp": "com.eurecom.calcite.SycldbTableScan", "table": ["ssb", "lineorder"],
               "inputs": []},
              {"id": "1", "relOp": "com.eurecom.calcite.SycldbFilter",
               "condition": {"op": {"name": "="}, "operands": [{"input": 5}, {"literal": "3"}]}}]},
])
def test_malformed_reljson_is_refused(bad):
    L = capi.lib()
    assert L.sdb_plan_check(json.dumps(bad).encode(), None, None, 0) == capi.SDB_ERR_INVALID
    assert capi.last_error()
