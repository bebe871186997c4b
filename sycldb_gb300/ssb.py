"""Seeded synthetic star-schema data (SSB shapes) for tests and benchmarks.

Every column comes from the counter-based generator of the native library
(``sdb_gen_uniform`` / ``sdb_gen_uniform_cpu``, SplitMix64 of
(seed, stream, row)), so host and device produce identical columns for any
row range.  The host generators take an optional ``gen`` object with the same
three functions (``uniform``, ``dates``, ``datekeys``) over numpy buffers:
the CPU checker supplies its own restatement through it, so that its legs
load nothing of the native library.  The public SSB dataset is not available offline; these columns
stand in for it with the distributions of the benchmark's configurations:

* lineorder (6,000,000 x SF rows): orderdate uniform over a 2,556-day
  calendar from 1992-01-01 encoded YYYYMMDD, discount 0..10, quantity 1..50,
  extendedprice 90,000..10,494,950, revenue 100,000..10,000,000, supplycost
  60,000..600,000, suppkey 1..2,000 x SF, partkey 1..54,000 x SF,
  custkey 1..30,000 x SF.
* supplier / customer: dense keys from 1, region 0..4, nation = 5 region + 0..4,
  city = 10 nation + 0..9.
* part (54,000 x SF rows): dense keys, category 0..24, brand1 =
  40 category + 0..39, mfgr = category / 5, size 1..50.
* ddate: one row per day of the 2,556-day calendar.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Iterable, Optional

import numpy as np

from . import capi

SEED = 20240601
NDAYS = 2556  # 1992-01-01 .. 1998-12-30
TABLE_IDS = {"lineorder": 0, "part": 1, "supplier": 2, "customer": 3, "ddate": 4}

# lineorder column index -> (kind, lo, hi); kinds: uniform, date, sfkey
# (uniform 1..base*SF).
LINEORDER = {
    0: ("sfkey", 1, 1_500_000),      # lo_orderkey
    1: ("uniform", 1, 7),            # lo_linenumber
    2: ("sfkey", 1, 30_000),         # lo_custkey
    3: ("sfkey", 1, 54_000),         # lo_partkey
    4: ("sfkey", 1, 2_000),          # lo_suppkey
    5: ("date", 0, NDAYS - 1),       # lo_orderdate
    6: ("uniform", 0, 4),            # lo_orderpriority
    7: ("uniform", 0, 0),            # lo_shippriority
    8: ("uniform", 1, 50),           # lo_quantity
    9: ("uniform", 90_000, 10_494_950),   # lo_extendedprice
    10: ("uniform", 90_000, 55_000_000),  # lo_ordtotalprice
    11: ("uniform", 0, 10),          # lo_discount
    12: ("uniform", 100_000, 10_000_000),  # lo_revenue
    13: ("uniform", 60_000, 600_000),  # lo_supplycost
    14: ("uniform", 0, 8),           # lo_tax
    15: ("date", 0, NDAYS - 1),      # lo_commitdate
    16: ("uniform", 0, 6),           # lo_shipmode
}

QUERY_COLUMNS = {
    "q1": (5, 8, 9, 11),        # filter-project-sum
    "q2": (5, 9, 11),           # filter + date join + group-by
    "star": (3, 4, 5, 12),      # three-way star join
    "flight3": (2, 4, 5, 12),   # customer, supplier, date joins -> three-key group-by
}


def stream_id(table: str, col: int, salt: int = 0) -> int:
    return (salt << 16) | (TABLE_IDS[table] << 8) | col


def fact_rows(sf: float) -> int:
    return int(round(6_000_000 * sf))


def dim_rows(table: str, sf: float) -> int:
    return {"supplier": int(round(2_000 * sf)), "part": int(round(54_000 * sf)),
            "customer": int(round(30_000 * sf)), "ddate": NDAYS}[table]


def _spec(col: int, sf: float):
    kind, lo, hi = LINEORDER[col]
    if kind == "sfkey":
        return "uniform", lo, max(lo, int(round(hi * sf)))
    return kind, lo, hi


class LibGen:
    """The native library's host generator (the default ``gen``)."""

    def uniform(self, a: np.ndarray, n: int, row0: int, seed: int, sid: int, lo: int, hi: int):
        capi.check(capi.lib().sdb_gen_uniform_cpu(a.ctypes.data, n, row0, seed, sid, lo, hi))

    def dates(self, a: np.ndarray, n: int, row0: int, seed: int, sid: int, ndays: int):
        capi.check(capi.lib().sdb_gen_dates_cpu(a.ctypes.data, n, row0, seed, sid, ndays))

    def datekeys(self, a: np.ndarray, n: int, day0: int):
        capi.check(capi.lib().sdb_gen_datekeys_cpu(a.ctypes.data, n, day0))


def _gen(gen):
    return gen if gen is not None else LibGen()


def gen_lineorder_host(n: int, cols: Iterable[int], sf: float, seed: int = SEED, row0: int = 0,
                       out: Optional[Dict[int, np.ndarray]] = None, salt: int = 0, gen=None) -> Dict[int, np.ndarray]:
    """Host columns (numpy int32; ``out`` may supply destination arrays,
    e.g. views of pinned tensors)."""
    g = _gen(gen)
    res = {}
    for c in cols:
        a = out[c] if out and c in out else np.empty(n, dtype=np.int32)
        assert a.dtype == np.int32 and a.size == n and a.flags["C_CONTIGUOUS"]
        kind, lo, hi = _spec(c, sf)
        sid = stream_id("lineorder", c, salt)
        if kind == "date":
            g.dates(a, n, row0, seed, sid, NDAYS)
        else:
            g.uniform(a, n, row0, seed, sid, lo, hi)
        res[c] = a
    return res


def gen_lineorder_device(n: int, cols: Iterable[int], sf: float, seed: int = SEED, row0: int = 0,
                         stream: int = 0, salt: int = 0):
    """Device columns (torch int32 CUDA tensors), identical to the host ones."""
    import torch

    L = capi.lib()
    res = {}
    for c in cols:
        t = torch.empty(n, dtype=torch.int32, device="cuda")
        kind, lo, hi = _spec(c, sf)
        sid = stream_id("lineorder", c, salt)
        if kind == "date":
            capi.check(L.sdb_gen_dates(t.data_ptr(), n, row0, seed, sid, NDAYS, stream or None))
        else:
            capi.check(L.sdb_gen_uniform(t.data_ptr(), n, row0, seed, sid, lo, hi, stream or None))
        res[c] = t
    return res


def _uniform(table: str, col: int, n: int, lo: int, hi: int, seed: int, salt: int = 0, gen=None) -> np.ndarray:
    a = np.empty(n, dtype=np.int32)
    _gen(gen).uniform(a, n, 0, seed, stream_id(table, col, salt), lo, hi)
    return a


def gen_geo_dim(table: str, n: int, seed: int = SEED, gen=None) -> Dict[int, np.ndarray]:
    """supplier / customer: key, city(3), nation(4), region(5)."""
    key = np.arange(1, n + 1, dtype=np.int32)
    region = _uniform(table, 5, n, 0, 4, seed, gen=gen)
    nation = (region * 5 + _uniform(table, 4, n, 0, 4, seed, gen=gen)).astype(np.int32)
    city = (nation * 10 + _uniform(table, 3, n, 0, 9, seed, gen=gen)).astype(np.int32)
    return {0: key, 3: city, 4: nation, 5: region}


def gen_part(n: int, seed: int = SEED, gen=None) -> Dict[int, np.ndarray]:
    key = np.arange(1, n + 1, dtype=np.int32)
    category = _uniform("part", 3, n, 0, 24, seed, gen=gen)
    brand = (category * 40 + _uniform("part", 4, n, 0, 39, seed, gen=gen)).astype(np.int32)
    mfgr = (category // 5).astype(np.int32)
    size = _uniform("part", 7, n, 1, 50, seed, gen=gen)
    return {0: key, 2: mfgr, 3: category, 4: brand, 7: size}


def gen_ddate(n: int = NDAYS, gen=None) -> Dict[int, np.ndarray]:
    key = np.empty(n, dtype=np.int32)
    _gen(gen).datekeys(key, n, 0)
    days = np.datetime64("1992-01-01") + np.arange(n)
    year = (key // 10000).astype(np.int32)
    month = (key // 100 % 100).astype(np.int32)
    dom = (key % 100).astype(np.int32)
    jan1 = days.astype("datetime64[Y]").astype("datetime64[D]")
    doy = ((days - jan1).astype(np.int64) + 1).astype(np.int32)
    dow = (((days.astype(np.int64) + 3) % 7) + 1).astype(np.int32)  # 1 = Monday
    return {0: key, 4: year, 5: (year * 100 + month).astype(np.int32), 7: dow, 8: dom, 9: doy, 10: month,
            11: ((doy - 1) // 7 + 1).astype(np.int32)}


def gen_dims(sf: float, seed: int = SEED, gen=None) -> Dict[str, Dict[int, np.ndarray]]:
    return {
        "supplier": gen_geo_dim("supplier", dim_rows("supplier", sf), seed, gen=gen),
        "customer": gen_geo_dim("customer", dim_rows("customer", sf), seed, gen=gen),
        "part": gen_part(dim_rows("part", sf), seed, gen=gen),
        "ddate": gen_ddate(gen=gen),
    }


def write_columnar(directory: str, tables: Dict[str, Dict[int, np.ndarray]]):
    """Writes tables in the reference's columnar layout: one raw int32 file
    per column, ``directory/<NAME><i>`` with the table's base name
    upper-cased (what ``Engine.load_dir`` and the reference's loader read)."""
    import os

    os.makedirs(directory, exist_ok=True)
    for name, cols in tables.items():
        base = name.split("@", 1)[0].upper()
        for c, a in cols.items():
            np.ascontiguousarray(a, dtype=np.int32).tofile(os.path.join(directory, "%s%d" % (base, c)))
