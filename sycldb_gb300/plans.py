"""Plan builders in the shape of the reference's Thrift PlanResult
(server/thrift/calciteserver.thrift:22-80), as JSON-ready dicts.

Calcite (the reference's planner) is not available offline, so the plans for
the benchmark configurations are written by hand in the shape the reference's
executor accepts (executor/ddor_executor.cpp:105-216): FILTER / PROJECT /
AGGREGATE / SORT consume the node just before them, JOIN takes the fact
side as input 0, ranges are SEARCH nodes with a one-range Sarg, dimensions
that contribute no output column join with joinType "semi".
"""
from __future__ import annotations

from typing import List, Sequence

NCOLS = {"lineorder": 17, "part": 9, "supplier": 7, "customer": 8, "ddate": 17}


# ------------------------------------------------------------------ expressions
def col(i: int, name: str = None) -> dict:
    return {"exprType": "COLUMN", "input": int(i), "name": name or "$%d" % i}


def lit(v: int) -> dict:
    return {"exprType": "LITERAL", "literal": {"literalOption": "LITERAL", "value": int(v)}}


def sarg_range(lo: int, hi: int) -> dict:
    return {"exprType": "LITERAL", "literal": {"literalOption": "RANGE", "rangeSet": [["[..]", str(lo), str(hi)]]}}


def sarg_points(a: int, b: int) -> dict:
    return {"exprType": "LITERAL",
            "literal": {"literalOption": "RANGE", "rangeSet": [["singleton", str(a)], ["singleton", str(b)]]}}


def expr(op: str, *operands) -> dict:
    return {"exprType": "EXPR", "op": op, "operands": list(operands)}


def search(c: int, lo: int, hi: int) -> dict:
    return expr("SEARCH", col(c), sarg_range(lo, hi))


def search_points(c: int, a: int, b: int) -> dict:
    return expr("SEARCH", col(c), sarg_points(a, b))


def AND(*xs) -> dict:
    return expr("AND", *xs)


def OR(*xs) -> dict:
    return expr("OR", *xs)


# ------------------------------------------------------------------ rel nodes
class PlanBuilder:
    def __init__(self):
        self.rels: List[dict] = []

    def _add(self, node: dict) -> int:
        node["id"] = len(self.rels)
        self.rels.append(node)
        return node["id"]

    def scan(self, table: str) -> int:
        return self._add({"relOp": "TABLE_SCAN", "tables": ["ssb", table], "inputs": []})

    def filter(self, cond: dict) -> int:
        return self._add({"relOp": "FILTER", "condition": cond})

    def join(self, left: int, right: int, left_col: int, right_col_abs: int, join_type: str = "inner") -> int:
        return self._add({"relOp": "JOIN", "inputs": [left, right],
                          "condition": expr("=", col(left_col), col(right_col_abs)), "joinType": join_type})

    def project(self, exprs: Sequence[dict]) -> int:
        return self._add({"relOp": "PROJECT", "fields": ["$f%d" % i for i in range(len(exprs))],
                          "exprs": list(exprs)})

    def aggregate(self, group: Sequence[int], operand: int, agg: str = "SUM") -> int:
        return self._add({"relOp": "AGGREGATE", "group": list(group),
                          "aggs": [{"agg": agg, "operands": [operand], "name": "$f%d" % len(group),
                                    "type": "BIGINT", "distinct": False}]})

    def sort(self, fields: Sequence[int]) -> int:
        return self._add({"relOp": "SORT", "collation": [{"field": f, "direction": "ASCENDING", "nulls": "LAST"}
                                                         for f in fields]})

    def plan(self) -> dict:
        return {"rels": self.rels}


def _t(name: str, tag) -> str:
    return name if tag is None else "%s@%s" % (name, tag)


# ------------------------------------------------------------------ configurations
def plan_filter_sum(year: int, disc_lo: int = 1, disc_hi: int = 3, qty_lt: int = 25, fact_tag=None) -> dict:
    """Filter-project-aggregate on the fact table: orderdate within one year
    AND discount in [disc_lo, disc_hi] AND quantity < qty_lt; SUM(extendedprice *
    discount)."""
    b = PlanBuilder()
    b.scan(_t("lineorder", fact_tag))
    b.filter(AND(search(5, year * 10000 + 101, year * 10000 + 1231), search(11, disc_lo, disc_hi),
                 expr("<", col(8), lit(qty_lt))))
    b.project([expr("*", col(9), col(11))])
    b.aggregate([], 0)
    return b.plan()


def plan_date_join(year0: int, disc_lo: int = 4, disc_hi: int = 6, fact_tag=None) -> dict:
    """Fact filter (discount) + join with a filtered date dimension (year in
    [year0, year0+1]), group by year, SUM(extendedprice * discount)."""
    b = PlanBuilder()
    f = b.scan(_t("lineorder", fact_tag))
    f = b.filter(search(11, disc_lo, disc_hi))
    d = b.scan("ddate")
    d = b.filter(search(4, year0, year0 + 1))
    j = b.join(f, d, 5, 17 + 0)
    b.project([col(17 + 4), expr("*", col(9), col(11))])
    b.aggregate([0], 1)
    b.sort([0])
    return b.plan()


def plan_star(region: int, category: int, year_lo: int = None, year_hi: int = None, brand_count: int = None,
              fact_tag=None) -> dict:
    """Three-way star join: supplier (region == r, semi join), part
    (category == c [, brand1 in the first brand_count brands of c]), date
    [, year range]; group by (year, brand1); SUM(revenue)."""
    b = PlanBuilder()
    f = b.scan(_t("lineorder", fact_tag))
    s = b.scan("supplier")
    s = b.filter(expr("==", col(5), lit(region)))
    j1 = b.join(f, s, 4, 17 + 0, "semi")                   # left now 17 + 7 = 24 columns
    p = b.scan("part")
    if brand_count is None:
        p = b.filter(expr("==", col(3), lit(category)))
    else:
        p = b.filter(AND(expr("==", col(3), lit(category)),
                         search(4, 40 * category, 40 * category + brand_count - 1)))
    j2 = b.join(j1, p, 3, 24 + 0)                           # p_brand1 -> 24 + 4 = 28; 33 columns
    d = b.scan("ddate")
    if year_lo is not None:
        d = b.filter(search(4, year_lo, year_hi))
    j3 = b.join(j2, d, 5, 33 + 0)                           # d_year -> 33 + 4 = 37; 50 columns
    b.project([col(37), col(28), col(12)])
    b.aggregate([0, 1], 2)
    b.sort([0, 1])
    return b.plan()


def plan_customer_supplier_date(region: int, year_lo: int = 1992, year_hi: int = 1997, city_points=None,
                                fact_tag=None) -> dict:
    """SSB flight-3 shape: lineorder joined with customer (region filter, or
    c_city in two points), supplier (same) and date (year range); group by
    (customer nation or city, supplier nation or city, d_year); SUM(lo_revenue).
    Three group-by keys, one from each dimension."""
    b = PlanBuilder()
    f = b.scan(_t("lineorder", fact_tag))
    c = b.scan("customer")
    if city_points:
        c = b.filter(search_points(3, city_points[0], city_points[1]))
    else:
        c = b.filter(expr("==", col(5), lit(region)))
    j1 = b.join(f, c, 2, 17 + 0)                           # customer -> 17..24
    s = b.scan("supplier")
    if city_points:
        s = b.filter(search_points(3, city_points[0], city_points[1]))
    else:
        s = b.filter(expr("==", col(5), lit(region)))
    j2 = b.join(j1, s, 4, 25 + 0)                          # supplier -> 25..31
    d = b.scan("ddate")
    d = b.filter(search(4, year_lo, year_hi))
    b.join(j2, d, 5, 32 + 0)                               # ddate -> 32..48
    key = 3 if city_points else 4                          # c/s_city or c/s_nation
    b.project([col(17 + key), col(25 + key), col(32 + 4), col(12)])
    b.aggregate([0, 1, 2], 3)
    b.sort([2, 0, 1])
    return b.plan()


def plan_profit(region: int, mfgr_points=(0, 1), fact_tag=None) -> dict:
    """SSB flight-4 shape: four joins -- customer (region, group by nation),
    supplier (region, semi join), part (p_mfgr in two points, semi join), date
    (group by year); SUM(lo_revenue - lo_supplycost)."""
    b = PlanBuilder()
    f = b.scan(_t("lineorder", fact_tag))
    c = b.scan("customer")
    c = b.filter(expr("==", col(5), lit(region)))
    j1 = b.join(f, c, 2, 17 + 0)                           # customer -> 17..24
    s = b.scan("supplier")
    s = b.filter(expr("==", col(5), lit(region)))
    j2 = b.join(j1, s, 4, 25 + 0, "semi")                  # supplier -> 25..31
    p = b.scan("part")
    p = b.filter(search_points(2, mfgr_points[0], mfgr_points[1]))
    j3 = b.join(j2, p, 3, 32 + 0, "semi")                  # part -> 32..40
    d = b.scan("ddate")
    b.join(j3, d, 5, 41 + 0)                               # ddate -> 41..57
    b.project([col(41 + 4), col(17 + 4), expr("-", col(12), col(13))])
    b.aggregate([0, 1], 2)
    b.sort([0, 1])
    return b.plan()
