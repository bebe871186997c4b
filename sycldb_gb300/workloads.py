"""Seeded multi-plan workloads: the batched form (many star-join plans over
fact partitions of uneven size) and the served form (a Poisson stream of mixed
plans over one resident star schema).

Everything here is deterministic in its seed; the data itself comes from the
counter-based generators of ``ssb`` (one salt per fact partition, so every
partition is an independent draw with the lineorder distributions).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import plans, ssb

# fact columns the star join reads: partkey, suppkey, orderdate, revenue
STAR_COLS = ssb.QUERY_COLUMNS["star"]


@dataclass
class StarParams:
    """Constants of one star-join plan (supplier region, part category, a
    year window and the number of brands of the category kept): it yields
    (year_hi - year_lo + 1) * brand_count groups at most."""
    region: int
    category: int
    year_lo: int
    year_hi: int
    brand_count: int

    @property
    def max_groups(self) -> int:
        return (self.year_hi - self.year_lo + 1) * self.brand_count

    def plan(self, fact_tag=None) -> dict:
        return plans.plan_star(self.region, self.category, self.year_lo, self.year_hi, self.brand_count,
                               fact_tag=fact_tag)


def draw_star_params(rng: np.random.Generator) -> StarParams:
    years = int(rng.integers(1, 8))
    y0 = int(rng.integers(1992, 1999 - years + 1))
    return StarParams(region=int(rng.integers(0, 5)), category=int(rng.integers(0, 25)), year_lo=y0,
                      year_hi=y0 + years - 1, brand_count=int(rng.integers(1, 41)))


@dataclass
class BatchWorkload:
    """n_plans star-join plans, plan p over its own fact partition
    ``lineorder@p`` of ``rows[p]`` rows."""
    rows: List[int]
    params: List[StarParams]
    dim_sf: float
    seed: int = ssb.SEED

    @property
    def n_plans(self) -> int:
        return len(self.rows)

    @property
    def total_rows(self) -> int:
        return int(sum(self.rows))

    def table(self, p: int) -> str:
        return "lineorder@%d" % p

    def plans(self) -> List[dict]:
        return [self.params[p].plan(fact_tag=p) for p in range(self.n_plans)]

    def algorithmic_bytes(self) -> int:
        """Every referenced column read once: 4 fact columns per row, plus the
        dimension columns each plan reads (supplier key+region, part
        key+category+brand1, date key+year)."""
        dims = (2 * ssb.dim_rows("supplier", self.dim_sf) + 3 * ssb.dim_rows("part", self.dim_sf) +
                2 * ssb.NDAYS) * 4
        return 16 * self.total_rows + dims * self.n_plans


def batch_workload(n_plans: int = 64, lo: int = 1_000_000, hi: int = 50_000_000, median: float = 7e6,
                   sigma: float = 1.0, dim_sf: float = 20, seed: int = ssb.SEED) -> BatchWorkload:
    """Partition sizes lognormal (median ``median``, log-sd ``sigma``) clipped
    to [lo, hi]; per-plan constants drawn from the same seed."""
    rng = np.random.default_rng([seed, 3])
    rows = np.clip(np.round(rng.lognormal(math.log(median), sigma, n_plans)), lo, hi).astype(np.int64)
    params = [draw_star_params(rng) for _ in range(n_plans)]
    return BatchWorkload([int(r) for r in rows], params, dim_sf, seed)


def load_batch_tables(eng, wl: BatchWorkload, device: bool = True, dims: Optional[dict] = None) -> Dict[str, dict]:
    """Registers the dimensions and every fact partition with ``eng``; fact
    partitions are generated on the device when ``device``.  Returns the
    tables (host numpy or device torch columns) keyed by name."""
    out = {}
    dims = dims if dims is not None else ssb.gen_dims(wl.dim_sf, wl.seed)
    for name in ("supplier", "part", "ddate"):
        eng.load_table(name, dims[name])
        out[name] = dims[name]
    for p, n in enumerate(wl.rows):
        if device:
            cols = ssb.gen_lineorder_device(n, STAR_COLS, wl.dim_sf, wl.seed, salt=p + 1)
        else:
            cols = ssb.gen_lineorder_host(n, STAR_COLS, wl.dim_sf, wl.seed, salt=p + 1)
        eng.load_table(wl.table(p), cols)
        out[wl.table(p)] = cols
    return out


# ---------------------------------------------------------------- served form

@dataclass
class Request:
    t: float          # arrival time, seconds from the start
    kind: str         # "filter_sum" | "date_join" | "star" | "batch_star"
    plan: dict = field(repr=False)


def _plan_of(kind: str, rng: np.random.Generator) -> dict:
    if kind == "filter_sum":
        y = int(rng.integers(1992, 1999))
        d = int(rng.integers(0, 9))
        return plans.plan_filter_sum(y, d, d + 2, int(rng.integers(10, 51)))
    if kind == "date_join":
        y = int(rng.integers(1992, 1998))
        d = int(rng.integers(0, 8))
        return plans.plan_date_join(y, d, d + 2)
    p = draw_star_params(rng)
    if kind == "star":
        return plans.plan_star(p.region, p.category)
    return p.plan()


def poisson_stream(rate_qps: float, n: int, mix=(("filter_sum", 0.25), ("date_join", 0.25), ("star", 0.25),
                                                  ("batch_star", 0.25)), seed: int = ssb.SEED) -> List[Request]:
    """n requests with exponential inter-arrival gaps of mean 1/rate_qps,
    plan shapes drawn from ``mix``."""
    rng = np.random.default_rng([seed, 4, int(rate_qps)])
    kinds = [k for k, _ in mix]
    w = np.array([p for _, p in mix], dtype=float)
    w /= w.sum()
    t = np.cumsum(rng.exponential(1.0 / rate_qps, n))
    out = []
    for i in range(n):
        k = kinds[int(rng.choice(len(kinds), p=w))]
        out.append(Request(float(t[i]), k, _plan_of(k, rng)))
    return out
