"""Autotuner for the fused fact-side pass.

The fused chain has eight kernel variants (``sdb_fused_chain_variant``):

  0/1/2  general interpreter, 4 / 8 / 16 rows per thread (items per thread)
  3      shape-specialised pass, every row through every op
  4      shape-specialised pass, rows compacted per warp after the first op,
         3-stage cp.async copy ring (3 blocks of 256 threads per SM)
  5      as 4 with a 2-stage ring (5 blocks per SM)
  6      as 5, surviving rows that do not fill a warp carried into the next tile
  7      as 6, and the rows that survive the first row-per-lane op compacted
         again (across lanes, in registers) so the later ops run on full warps

Block size is 256 threads throughout; the group-by tables are direct-address
(the reference's HASH is the identity on its range), so there is no load
factor to pick for the joins, and the shared-memory group table of the
specialised passes has a fixed 512-slot capacity.  The tuner times every
variant on the plan shapes of the benchmark at several fact sizes, picks the
fastest per tuning key -- (terminal, register class, kind of the chain's
first op, log2 rows bucket), the key of ``sdb_chain_tune_set_op`` -- and
writes the table as JSON.  ``load`` puts a
table into the library; ``Engine`` loads the default table for the device at
creation.

    python -m sycldb_gb300.autotune --out tuning.json [--sizes 1e6,4e6,...]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import time
from typing import Dict, Iterable, List, Optional

from . import capi, plans, ssb

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tuning", "gb300.json")
VARIANTS = (0, 1, 2, 3, 4, 5, 6, 7)
TERMINALS = {"flags": 0, "sum": 1, "groupby": 2}

OP_SEARCH_RANGE, OP_SEMI_PROBE = 1, 3  # SDB_OP_* kinds of a chain's first op

# benchmark plan shapes: (name, terminal, registers, first op, fact columns, plan builder)
SHAPES = [
    ("filter_sum", "sum", 1, OP_SEARCH_RANGE, ssb.QUERY_COLUMNS["q1"], lambda: plans.plan_filter_sum(1994)),
    ("date_join", "groupby", 2, OP_SEARCH_RANGE, ssb.QUERY_COLUMNS["q2"], lambda: plans.plan_date_join(1994)),
    ("star", "groupby", 2, OP_SEMI_PROBE, ssb.QUERY_COLUMNS["star"], lambda: plans.plan_star(2, 11)),
]


def rows_bucket(n: int) -> int:
    """log2 bucket of the library's tuning table: largest b with 2^b <= n."""
    return max(0, min(39, int(math.floor(math.log2(max(n, 1))))))


def load(table: dict) -> int:
    """Puts every entry of a tuning table into the library; returns how many.
    A measured bucket's choice also holds for the unmeasured buckets above
    it, up to the next measured one (the largest: up to the table's end), so
    sizes between and beyond the measured ones take their nearest smaller
    neighbour's variant instead of the library default."""
    L = capi.lib()
    entries = table.get("entries", [])
    by_key = {}
    for e in entries:
        by_key.setdefault((e["terminal"], e["nregs"], e.get("first_op", -1)), []).append(e)
    for (term, nregs, first_op), es in by_key.items():
        es = sorted(es, key=lambda e: e["rows_bucket"])
        for i, e in enumerate(es):
            hi = es[i + 1]["rows_bucket"] if i + 1 < len(es) else 40
            for b in range(e["rows_bucket"], hi):
                capi.check(L.sdb_chain_tune_set_op(TERMINALS[term], nregs, first_op, 1 << b, e["variant"]))
    return len(entries)


def load_default(path: Optional[str] = None) -> Optional[dict]:
    """Loads the committed table (if present); returns it."""
    path = path or os.environ.get("SYCLDB_TUNING", DEFAULT_TABLE)
    if not path or not os.path.exists(path):
        return None
    with open(path) as f:
        table = json.load(f)
    load(table)
    return table


def _time_variant(eng, plan, variant: int, reps: int) -> float:
    capi.force_chain_variant(variant)
    eng.execute(plan)  # warm
    ms = []
    for _ in range(reps):
        eng.execute(plan)
        st = eng.kernel_stats()
        ms.append(st["fused_chain"][1] if "fused_chain" in st else float("inf"))
    return statistics.median(ms)


def tune(sizes: Iterable[int] = (1 << 20, 1 << 22, 1 << 24, 1 << 26, 120_000_000), reps: int = 5,
         variants=VARIANTS, shapes=SHAPES, sf_dims: float = 20, log=print) -> dict:
    """Times every variant of every benchmark shape at each fact size on the
    current device and returns the tuning table."""
    import torch

    from .engine import Engine

    dims = ssb.gen_dims(sf_dims)
    cols = sorted({c for s in shapes for c in s[4]})
    timings: Dict[tuple, Dict[int, float]] = {}
    per_shape = []
    for n in sizes:
        fact = ssb.gen_lineorder_device(int(n), cols, sf_dims, salt=7)
        torch.cuda.synchronize()
        with Engine(fuse=True, profile=True) as eng:
            eng.load_table("lineorder", fact)
            for t in ("supplier", "part", "ddate"):
                eng.load_table(t, dims[t])
            for name, term, nregs, first_op, _, build in shapes:
                plan = build()
                res = {v: _time_variant(eng, plan, v, reps) for v in variants}
                key = (term, nregs, first_op, rows_bucket(int(n)))
                acc = timings.setdefault(key, {})
                for v, t in res.items():
                    acc[v] = acc.get(v, 0.0) + t
                per_shape.append({"shape": name, "rows": int(n), "ms": {str(v): t for v, t in res.items()}})
                log("%-10s rows=%-10d %s" % (name, n, " ".join("v%d=%.4f" % (v, t) for v, t in res.items())))
        del fact
        torch.cuda.empty_cache()
    capi.force_chain_variant(-1)
    entries = []
    for (term, nregs, first_op, b), acc in sorted(timings.items()):
        best = min(acc, key=acc.get)
        entries.append({"terminal": term, "nregs": nregs, "first_op": first_op, "rows_bucket": b, "variant": best,
                        "ms_sum": {str(v): t for v, t in acc.items()}})
    return {"device": torch.cuda.get_device_name(), "created": time.strftime("%Y-%m-%d %H:%M:%S"),
            "reps": reps, "sizes": [int(n) for n in sizes], "entries": entries, "measurements": per_shape}


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", required=True)
    ap.add_argument("--sizes", default="1048576,4194304,16777216,67108864,120000000")
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    from . import build

    build.build()
    table = tune([int(float(x)) for x in a.sizes.split(",")], reps=a.reps)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(table, f, indent=1)
    print("wrote %s (%d entries)" % (a.out, len(table["entries"])))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
