"""Independent naive evaluator (plain SQL semantics with numpy / dicts) for the
plan shapes of sycldb_gb300.plans.  It shares no code with the oracle's
executor restatement; the tests require both to agree.  Sums are int64
two's complement reported as uint64 (mod 2^64)."""
import numpy as np


def _u64(x: int) -> int:
    return x & 0xFFFFFFFFFFFFFFFF


def filter_sum(fact, year, disc_lo=1, disc_hi=3, qty_lt=25):
    d, q, p, c = fact[5], fact[8], fact[9], fact[11]
    m = (d >= year * 10000 + 101) & (d <= year * 10000 + 1231) & (c >= disc_lo) & (c <= disc_hi) & (q < qty_lt)
    prod = (p[m].astype(np.int64) * c[m].astype(np.int64))
    prod = ((prod + 2 ** 31) % 2 ** 32 - 2 ** 31)  # int32 multiply wraps
    return [(_u64(int(prod.sum())),)]


def date_join(fact, ddate, year0, disc_lo=4, disc_hi=6):
    year_of = dict(zip(ddate[0].tolist(), ddate[4].tolist()))
    c = fact[11]
    m = (c >= disc_lo) & (c <= disc_hi)
    out = {}
    for od, pr, dc in zip(fact[5][m].tolist(), fact[9][m].tolist(), c[m].tolist()):
        y = year_of.get(od)
        if y is None or not (year0 <= y <= year0 + 1):
            continue
        v = ((pr * dc + 2 ** 31) % 2 ** 32) - 2 ** 31
        out[y] = out.get(y, 0) + v
    return sorted((y, _u64(s)) for y, s in out.items())


def star(fact, supplier, part, ddate, region, category, year_lo=None, year_hi=None, brand_count=None):
    sup_ok = set(supplier[0][supplier[5] == region].tolist())
    pm = part[3] == category
    if brand_count is not None:
        pm &= (part[4] >= 40 * category) & (part[4] <= 40 * category + brand_count - 1)
    brand_of = dict(zip(part[0][pm].tolist(), part[4][pm].tolist()))
    dm = np.ones(ddate[0].size, bool)
    if year_lo is not None:
        dm = (ddate[4] >= year_lo) & (ddate[4] <= year_hi)
    year_of = dict(zip(ddate[0][dm].tolist(), ddate[4][dm].tolist()))
    s_ok = np.isin(fact[4], np.fromiter(sup_ok, dtype=np.int64, count=len(sup_ok))) if sup_ok else np.zeros(fact[4].size, bool)
    p_ok = np.isin(fact[3], np.fromiter(brand_of.keys(), dtype=np.int64, count=len(brand_of))) if brand_of else np.zeros(fact[3].size, bool)
    m = s_ok & p_ok
    out = {}
    for pk, od, rev in zip(fact[3][m].tolist(), fact[5][m].tolist(), fact[12][m].tolist()):
        y = year_of.get(od)
        if y is None:
            continue
        k = (y, brand_of[pk])
        out[k] = out.get(k, 0) + rev
    return sorted((y, b, _u64(s)) for (y, b), s in out.items())
