"""Writes the hand-made Calcite RelJson plans of this folder (SSB q1.1, q2.1,
q3.1, shaped on queries/transformed/q11.sql, q21.sql, q31.sql of the
reference).  They follow the dialect that the reference's
SycldbJsonConverter reads (server/src/main/java/com/eurecom/calcite/
SycldbJsonConverter.java:31-163): planner class names as relOp, "table",
string ids and inputs, {"name", "kind", "syntax"} operators, bare-number
literals and Sarg rangeSets, {"type", "nullable"} types.  No plan captured
from Calcite exists in the reference, so the join order and the projections
are the ones the reference executor accepts (fact table on the left of every
join, dimension filters before their join, semi joins for dimensions that
contribute no output column).

    python tests/golden/reljson/make_reljson.py
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def T(nullable=False, t="INTEGER"):
    return {"type": t, "nullable": nullable}


def col(i):
    return {"input": i, "name": "$%d" % i}


def lit(v):
    return {"literal": v, "type": T()}


def call(name, kind, *ops, syntax="BINARY"):
    return {"op": {"name": name, "kind": kind, "syntax": syntax}, "operands": list(ops)}


def search(c, lo, hi):
    sarg = {"literal": {"rangeSet": [["[..]", str(lo), str(hi)]], "nullAs": "UNKNOWN"}, "type": T()}
    return call("SEARCH", "SEARCH", col(c), sarg, syntax="INTERNAL")


def eq(a, b):
    return call("=", "EQUALS", a, b)


def scan(i, t):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbTableScan", "table": ["ssb", t], "inputs": []}


def filt(i, c):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbFilter", "condition": c}


def join(i, left, right, c, jt):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbJoin", "condition": c, "joinType": jt,
            "inputs": [str(left), str(right)]}


def proj(i, fields, exprs):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbProject", "fields": fields, "exprs": exprs}


def agg(i, group, op, name):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbAggregate", "group": group,
            "aggs": [{"agg": {"name": "SUM", "kind": "SUM", "syntax": "FUNCTION"}, "type": T(True, "BIGINT"),
                      "distinct": False, "operands": [op], "name": name}]}


def sort(i, coll):
    return {"id": str(i), "relOp": "com.eurecom.calcite.SycldbSort",
            "collation": [{"field": f, "direction": d, "nulls": "LAST"} for f, d in coll]}


def plans():
    q11 = {"rels": [
        scan(0, "lineorder"),
        filt(1, call("AND", "AND", search(5, 19930101, 19940101), search(11, 1, 3),
                     call("<", "LESS_THAN", col(8), lit(25)))),
        proj(2, ["$f0"], [call("*", "TIMES", col(9), col(11))]),
        agg(3, [], 0, "REVENUE"),
    ]}
    # lineorder (17 columns) x part (9) -> 26, x supplier (7, semi) -> 33, x ddate (17) -> 50
    q21 = {"rels": [
        scan(0, "lineorder"),
        scan(1, "part"),
        filt(2, eq(col(3), lit(1))),
        join(3, 0, 2, eq(col(3), col(17)), "inner"),
        scan(4, "supplier"),
        filt(5, eq(col(5), lit(1))),
        join(6, 3, 5, eq(col(4), col(26)), "semi"),
        scan(7, "ddate"),
        join(8, 6, 7, eq(col(5), col(33)), "inner"),
        proj(9, ["d_year", "p_brand1", "lo_revenue"], [col(37), col(21), col(12)]),
        agg(10, [0, 1], 2, "EXPR$0"),
        sort(11, [(0, "ASCENDING"), (1, "ASCENDING")]),
    ]}
    # lineorder (17) x customer (8) -> 25, x supplier (7) -> 32, x ddate (17) -> 49
    q31 = {"rels": [
        scan(0, "lineorder"),
        scan(1, "customer"),
        filt(2, eq(col(5), lit(2))),
        join(3, 0, 2, eq(col(2), col(17)), "inner"),
        scan(4, "supplier"),
        filt(5, eq(col(5), lit(2))),
        join(6, 3, 5, eq(col(4), col(25)), "inner"),
        scan(7, "ddate"),
        filt(8, search(4, 1992, 1997)),
        join(9, 6, 8, eq(col(5), col(32)), "inner"),
        proj(10, ["c_nation", "s_nation", "d_year", "lo_revenue"], [col(21), col(29), col(36), col(12)]),
        agg(11, [0, 1, 2], 3, "REVENUE"),
        sort(12, [(2, "ASCENDING"), (3, "DESCENDING")]),
    ]}
    return {"q11": q11, "q21": q21, "q31": q31}


if __name__ == "__main__":
    for name, q in plans().items():
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(q, f, indent=1)
            f.write("\n")
