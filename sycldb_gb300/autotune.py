"""Autotuner for the fused fact-side pass.

The fused chain has nine kernel variants (``sdb_fused_chain_variant``):

  0/1/2  general interpreter, 4 / 8 / 16 rows per thread (items per thread)
  3      shape-specialised pass, every row through every op
  4      shape-specialised pass, rows compacted per warp after the first op,
         3-stage cp.async copy ring (3 blocks of 256 threads per SM)
  5      as 4 with a 2-stage ring (5 blocks per SM)
  6      as 5, surviving rows that do not fill a warp carried into the next tile
  7      as 6, and the rows that survive the first row-per-lane op compacted
         again (across lanes, in registers) so the later ops run on full warps
  8      as 7, and the columns that only the ops after that second compaction
         read are not staged: each surviving row loads them by row number

The fused passes keep 256 threads per block: their copy ring, per-warp row
lists and tile shape (256 x 4 rows) are laid out for it, and the variants
above are the measured alternatives.  The operator-at-a-time kernels (K1-K16,
the unfused path) take a tuned launch shape instead: threads per block
(128 / 256 / 512) and resident blocks per SM of their grid-stride grid, per
kernel and log2 rows bucket (``sdb_op_tune_set``; ``op_entries`` of the
table).  The join tables are direct-address (the reference's HASH is the
identity on its range, kernels/join.hpp:11-15), so there is no load factor
to pick; the open-addressing tables taken for sparse key ranges have a fixed
sizing rule (the smallest power of two at least twice the build rows, load
at most 0.5), chosen with the engine's ``join_tables`` option rather than
tuned; and the shared-memory group table of the specialised passes has a
fixed 512-slot capacity.  The tuner times every
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
VARIANTS = (0, 1, 2, 3, 4, 5, 6, 7, 8)
TERMINALS = {"flags": 0, "sum": 1, "groupby": 2}

OP_SEARCH_RANGE, OP_SEMI_PROBE, OP_FULL_PROBE = 1, 3, 4  # SDB_OP_* kinds of a chain's first op

# benchmark plan shapes: (name, terminal, registers, first op, fact columns, plan builder)
SHAPES = [
    ("filter_sum", "sum", 1, OP_SEARCH_RANGE, ssb.QUERY_COLUMNS["q1"], lambda: plans.plan_filter_sum(1994)),
    ("date_join", "groupby", 2, OP_SEARCH_RANGE, ssb.QUERY_COLUMNS["q2"], lambda: plans.plan_date_join(1994)),
    ("star", "groupby", 2, OP_SEMI_PROBE, ssb.QUERY_COLUMNS["star"], lambda: plans.plan_star(2, 11)),
    # three full probes (the fused pass tests the supplier table's bitmap first;
    # the tuning key is the chain as the executor hands it over)
    ("flight3", "groupby", 3, OP_FULL_PROBE, ssb.QUERY_COLUMNS["flight3"],
     lambda: plans.plan_customer_supplier_date(2)),
]


def rows_bucket(n: int) -> int:
    """log2 bucket of the library's tuning table: largest b with 2^b <= n."""
    return max(0, min(39, int(math.floor(math.log2(max(n, 1))))))


OP_BLOCKS = (128, 256, 512)
OP_PER_SM = (2, 4, 8, 16)
LOAD_FACTOR_NOTE = ("no load-factor axis: the join tables are direct-address over their key range "
                    "(kernels/join.hpp:11-15), so their size is fixed by the build column's min/max; "
                    "the open-addressing tables of sparse key ranges take the smallest power of two "
                    "at least twice the build rows (load at most 0.5), a fixed rule")


def load_ops(table: dict) -> int:
    """Puts the operator kernels' launch shapes of a tuning table into the
    library (a measured bucket's shape also holds for the buckets above it up
    to the next measured one); returns how many entries."""
    L = capi.lib()
    by_op = {}
    for e in table.get("op_entries", []):
        by_op.setdefault(e["kernel"], []).append(e)
    for name, es in by_op.items():
        k = capi.OP_KERNELS.index(name)
        es = sorted(es, key=lambda e: e["rows_bucket"])
        for i, e in enumerate(es):
            hi = es[i + 1]["rows_bucket"] if i + 1 < len(es) else 40
            for b in range(e["rows_bucket"], hi):
                capi.check(L.sdb_op_tune_set(k, 1 << b, e["block"], e["blocks_per_sm"]))
    return len(table.get("op_entries", []))


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
    load_ops(table)
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
            for t in ("supplier", "customer", "part", "ddate"):
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


def _op_calls(n: int):
    """One call per operator kernel over n rows of device buffers (seeded,
    the selectivities of the benchmark: a fifth of the rows live)."""
    import ctypes

    import torch

    L = capi.lib()
    g = torch.Generator(device="cuda").manual_seed(5)
    dev = lambda t: t.data_ptr()  # noqa: E731
    col = torch.randint(0, 1_000_000, (n,), dtype=torch.int32, device="cuda", generator=g)
    col2 = torch.randint(0, 1_000_000, (n,), dtype=torch.int32, device="cuda", generator=g)
    fl = (torch.rand(n, device="cuda", generator=g) < 0.2).to(torch.uint8)
    out8 = torch.empty(n, dtype=torch.uint8, device="cuda")
    out32 = torch.empty(n, dtype=torch.int32, device="cuda")
    acc = torch.zeros(2, dtype=torch.int64, device="cuda")
    ht_len = 1 << 20
    key = torch.randint(0, ht_len, (n,), dtype=torch.int32, device="cuda", generator=g)
    ht8 = torch.zeros(ht_len, dtype=torch.uint8, device="cuda")
    ht2 = torch.zeros(2 * ht_len, dtype=torch.int32, device="cuda")
    occ = (torch.rand(n, device="cuda", generator=g) < 0.2).to(torch.int32)
    ids = torch.arange(0, n, 5, dtype=torch.int32, device="cuda")
    cnt = torch.tensor([ids.numel()], dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    keep = [col, col2, fl, out8, out32, acc, key, ht8, ht2, occ, ids, cnt]
    calls = {
        "fill_u8": lambda: L.sdb_fill_u8(dev(out8), n, 1, s),
        "select_lit": lambda: L.sdb_select_lit(dev(col), 500_000, 2, 1, dev(fl), dev(out8), n, s),
        "select_cols": lambda: L.sdb_select_cols(dev(col), dev(col2), 2, 1, dev(fl), dev(out8), n, s),
        "logical": lambda: L.sdb_logical(1, dev(fl), dev(out8), dev(out8), n, s),
        "fill_i32": lambda: L.sdb_fill_i32(dev(out32), 3, n, s),
        "binop": lambda: L.sdb_binop_cc(dev(out32), dev(col), dev(col2), 0, dev(fl), n, s),
        "sum": lambda: L.sdb_sum_i32_u64(dev(col), dev(fl), n, dev(acc), s),
        "count_flags": lambda: L.sdb_count_flags(dev(fl), n, dev(acc), s),
        "min_max": lambda: L.sdb_min_max_i32(dev(col), n, dev(acc), s),
        "occ_to_flags": lambda: L.sdb_occ_to_flags(dev(occ), dev(out8), n, s),
        "build_keys": lambda: L.sdb_ht_build_keys(dev(key), dev(fl), n, dev(ht8), 0, ht_len, s),
        "probe_semi": lambda: L.sdb_probe_semi(dev(key), dev(fl), dev(out8), n, dev(ht8), 0, ht_len - 1, s),
        "build_kv": lambda: L.sdb_ht_build_kv(dev(key), dev(col), dev(fl), n, dev(ht2), 0, ht_len, s),
        "probe_full": lambda: L.sdb_probe_full(dev(key), dev(out32), dev(fl), dev(out8), n, dev(ht2), 0, ht_len - 1, s),
        "gather": lambda: L.sdb_gather_i32(dev(col), dev(ids), dev(cnt), dev(out32), ids.numel(), s),
    }
    return calls, keep


def tune_ops(sizes: Iterable[int] = (1 << 20, 1 << 22, 1 << 24, 1 << 26), reps: int = 7, log=print) -> List[dict]:
    """Times every launch shape (threads per block x resident blocks per SM)
    of every operator kernel at each size; returns the fastest per (kernel,
    log2 rows bucket)."""
    import torch

    L = capi.lib()
    entries = []
    for n in sizes:
        calls, keep = _op_calls(int(n))
        b = rows_bucket(int(n))
        for name, call in calls.items():
            k = capi.OP_KERNELS.index(name)
            res = {}
            for blk in OP_BLOCKS:
                for per in OP_PER_SM:
                    if blk * per > 2048:
                        continue
                    capi.check(L.sdb_op_tune_set(k, int(n), blk, per))
                    capi.check(call())
                    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                    ts = []
                    for _ in range(reps):
                        ev[0].record()
                        capi.check(call())
                        ev[1].record()
                        ev[1].synchronize()
                        ts.append(ev[0].elapsed_time(ev[1]))
                    res[(blk, per)] = statistics.median(ts)
            capi.check(L.sdb_op_tune_set(k, int(n), 0, 0))
            (blk, per), best = min(res.items(), key=lambda kv: kv[1])
            entries.append({"kernel": name, "rows_bucket": b, "block": blk, "blocks_per_sm": per, "ms": best,
                            "ms_default": res.get((256, 4 if name in ("sum", "count_flags", "min_max") else 8))})
            log("%-12s rows=%-10d best %d x %d  %.4f ms (default %.4f)" % (name, n, blk, per, best,
                                                                           entries[-1]["ms_default"]))
        del calls, keep
        torch.cuda.empty_cache()
    return entries


def main(argv: Optional[List[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", required=True)
    ap.add_argument("--sizes", default="1048576,4194304,16777216,67108864,120000000")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--ops-only", action="store_true",
                    help="tune only the operator kernels' launch shapes and merge them into an existing --out table")
    a = ap.parse_args(argv)
    from . import build

    build.build()
    if a.ops_only and os.path.exists(a.out):
        with open(a.out) as f:
            table = json.load(f)
    else:
        table = tune([int(float(x)) for x in a.sizes.split(",")], reps=a.reps)
    table["op_entries"] = tune_ops()
    table["op_note"] = LOAD_FACTOR_NOTE
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(table, f, indent=1)
    print("wrote %s (%d entries)" % (a.out, len(table["entries"])))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
