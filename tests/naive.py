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


# ---------------------------------------------------------------------------
# Vectorised forms of the same three shapes, for full-size checks (hundreds of
# millions of fact rows): lookup arrays over each dimension key range instead
# of dicts, exact int64 group sums.  They must give the loops' rows (checked
# on CPU at small scale).

def _exact_sums(idx: np.ndarray, v: np.ndarray, ngroups: int):
    """Exact int64 sums of v per group index: v = hi * 2^24 + lo with
    0 <= lo < 2^24, each part summed with bincount in float64, whose partial
    sums stay integers below 2^53 for fewer than 2^29 rows per call."""
    v = v.astype(np.int64)
    out = np.zeros(ngroups, dtype=object)
    step = 1 << 28
    for s in range(0, idx.size, step):
        i, w = idx[s:s + step], v[s:s + step]
        lo = (w & 0xFFFFFF).astype(np.float64)
        hi = (w >> 24).astype(np.float64)
        slo = np.bincount(i, weights=lo, minlength=ngroups)
        shi = np.bincount(i, weights=hi, minlength=ngroups)
        cnt = np.bincount(i, minlength=ngroups)
        for g in np.flatnonzero(cnt):
            out[g] += int(shi[g]) * (1 << 24) + int(slo[g])
    return out, np.bincount(idx, minlength=ngroups) if idx.size else np.zeros(ngroups, np.int64)


def _lut(keys: np.ndarray, vals: np.ndarray, keep: np.ndarray):
    """key -> value lookup over [min key, max key] of the whole key column;
    -1 where the key is absent or filtered out (values are non-negative)."""
    lo, hi = int(keys.min()), int(keys.max())
    t = np.full(hi - lo + 1, -1, dtype=np.int64)
    t[keys[keep].astype(np.int64) - lo] = vals[keep]
    return t, lo, hi


def _probe(t, lo, hi, k: np.ndarray):
    k = k.astype(np.int64)
    inr = (k >= lo) & (k <= hi)
    out = np.full(k.size, -1, dtype=np.int64)
    out[inr] = t[k[inr] - lo]
    return out


def _wrap32(x: np.ndarray) -> np.ndarray:
    return ((x.astype(np.int64) + 2 ** 31) % 2 ** 32) - 2 ** 31


def date_join_vec(fact, ddate, year0, disc_lo=4, disc_hi=6):
    keep = (ddate[4] >= year0) & (ddate[4] <= year0 + 1)
    t, lo, hi = _lut(ddate[0], ddate[4].astype(np.int64), keep)
    c = fact[11]
    m = (c >= disc_lo) & (c <= disc_hi)
    y = _probe(t, lo, hi, fact[5][m])
    sel = y >= 0
    v = _wrap32(fact[9][m][sel].astype(np.int64) * c[m][sel].astype(np.int64))
    y = y[sel]
    if not y.size:
        return []
    y0 = int(y.min())
    sums, cnt = _exact_sums(y - y0, v, int(y.max()) - y0 + 1)
    return [(y0 + g, _u64(int(sums[g]))) for g in np.flatnonzero(cnt)]


def star_vec(fact, supplier, part, ddate, region, category, year_lo=None, year_hi=None, brand_count=None):
    st, slo, shi = _lut(supplier[0], np.ones(supplier[0].size, np.int64), supplier[5] == region)
    pm = part[3] == category
    if brand_count is not None:
        pm &= (part[4] >= 40 * category) & (part[4] <= 40 * category + brand_count - 1)
    pt, plo, phi = _lut(part[0], part[4].astype(np.int64), pm)
    dm = np.ones(ddate[0].size, bool)
    if year_lo is not None:
        dm = (ddate[4] >= year_lo) & (ddate[4] <= year_hi)
    dt, dlo, dhi = _lut(ddate[0], ddate[4].astype(np.int64), dm)
    idx = np.flatnonzero(_probe(st, slo, shi, fact[4]) >= 0)
    brand = _probe(pt, plo, phi, fact[3][idx])
    idx, brand = idx[brand >= 0], brand[brand >= 0]
    year = _probe(dt, dlo, dhi, fact[5][idx])
    idx, brand, year = idx[year >= 0], brand[year >= 0], year[year >= 0]
    if not idx.size:
        return []
    comp = year * 100000 + brand
    uniq, inv = np.unique(comp, return_inverse=True)
    sums, _ = _exact_sums(inv.ravel(), fact[12][idx].astype(np.int64), uniq.size)
    return sorted((int(u // 100000), int(u % 100000), _u64(int(s))) for u, s in zip(uniq, sums))


def filter_sum_vec(fact, year, disc_lo=1, disc_hi=3, qty_lt=25):
    d, q, p, c = fact[5], fact[8], fact[9], fact[11]
    m = (d >= year * 10000 + 101) & (d <= year * 10000 + 1231) & (c >= disc_lo) & (c <= disc_hi) & (q < qty_lt)
    prod = _wrap32(p[m].astype(np.int64) * c[m].astype(np.int64))
    sums, _ = _exact_sums(np.zeros(prod.size, np.int64), prod, 1)
    return [(_u64(int(sums[0])),)]
