"""Generates the committed golden vectors under tests/golden/.

* kernels.npz + kernels.json: seeded inputs and the outputs of the
  REFERENCE's own kernel functors (kernels/*.hpp compiled against the host SYCL
  shim, oracle/_ref) for every kernel type of the C ABI.
* plans.json: plans of the benchmark shapes on small seeded datasets, with the
  expected result rows from the oracle executor (its kernels pinned to the
  reference functors), cross-checked against the independent naive evaluator,
  and checksums of the generated columns.

Run from the repository root, where the reference checkout is present:
    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402

build_oracle.build_oracle()
assert build_oracle.build_ref(), "the reference checkout is needed to generate golden vectors"

from sycldb_gb300 import build, plans  # noqa: E402

build.build()

from tests import datasets, kernel_cases as kc, naive, refkern as R  # noqa: E402


def kernel_cases():
    L = R.lib()
    arrays = {}
    cases = []

    def add(name, kernel, params, ins, outs):
        for k, v in ins.items():
            arrays["%s/in/%s" % (name, k)] = v
        for k, v in outs.items():
            arrays["%s/out/%s" % (name, k)] = v
        cases.append({"name": name, "kernel": kernel, "params": params,
                      "inputs": sorted(ins), "outputs": sorted(outs)})

    n = 515
    for cmp in range(6):
        for logic in range(3):
            rng = np.random.default_rng(1000 + cmp * 3 + logic)
            col, fin = kc.col_wide(rng, n), kc.flags(rng, n)
            col[::7] = 12345
            out = np.empty(n, np.uint8)
            L.ref_select_lit(R.ptr(col), 12345, cmp, logic, R.ptr(fin), R.ptr(out), n)
            add("select_lit_%d_%d" % (cmp, logic), "select_lit", {"v": 12345, "cmp": cmp, "logic": logic},
                {"col": col, "in": fin}, {"out": out})
            b = kc.col_wide(rng, n)
            b[::3] = col[::3]
            out2 = np.empty(n, np.uint8)
            L.ref_select_cols(R.ptr(col), R.ptr(b), cmp, logic, R.ptr(fin), R.ptr(out2), n)
            add("select_cols_%d_%d" % (cmp, logic), "select_cols", {"cmp": cmp, "logic": logic},
                {"a": col, "b": b, "in": fin}, {"out": out2})
    for logic in range(3):
        rng = np.random.default_rng(2000 + logic)
        fin, loc = kc.flags(rng, n), kc.flags(rng, n)
        out = np.empty(n, np.uint8)
        L.ref_logical(logic, R.ptr(fin), R.ptr(loc), R.ptr(out), n)
        add("logical_%d" % logic, "logical", {"logic": logic}, {"in": fin, "local": loc}, {"out": out})
    out = np.zeros(n, np.int32)
    L.ref_fill_i32(R.ptr(out), -77, n)
    add("fill_i32", "fill_i32", {"v": -77}, {}, {"out": out})
    for op in range(4):
        rng = np.random.default_rng(3000 + op)
        x, y = kc.col_wide(rng, n), kc.col_wide(rng, n)
        if op == 1:
            y = kc.divisor(rng, n)
            x = kc.numerators_for(x, y)
        fl = kc.flags(rng, n)
        for mode in ("cc", "lc", "cl"):
            res = np.full(n, 99, np.int32)
            la, lb = -1000003, 7
            if mode == "cc":
                L.ref_binop_cc(R.ptr(res), R.ptr(x), R.ptr(y), op, R.ptr(fl), n)
            elif mode == "lc":
                L.ref_binop_lc(R.ptr(res), la, R.ptr(y), op, R.ptr(fl), n)
            else:
                L.ref_binop_cl(R.ptr(res), R.ptr(x), lb, op, R.ptr(fl), n)
            add("binop_%s_%d" % (mode, op), "binop_" + mode, {"op": op, "la": la, "lb": lb},
                {"a": x, "b": y, "flags": fl, "res0": np.full(n, 99, np.int32)}, {"res": res})
    for p in (0.0, 0.3, 1.0):
        rng = np.random.default_rng(4000 + int(p * 10))
        col, fl = kc.col_wide(rng, 2053), kc.flags(rng, 2053, p)
        acc = np.array([5], np.uint64)
        L.ref_sum_i32_u64(R.ptr(col), R.ptr(fl), 2053, R.ptr(acc))
        add("sum_%d" % int(p * 10), "sum", {"acc0": 5}, {"col": col, "flags": fl}, {"acc": acc})
    for g in (1, 2, 3):
        rng = np.random.default_rng(5000 + g)
        m = 5003
        ranges = [(1992, 1998), (0, 99), (-2, 2)][:g]
        keys = [rng.integers(lo, hi + 1, m).astype(np.int32) for lo, hi in ranges]
        mins = np.array([r[0] for r in ranges], np.int32)
        maxs = np.array([r[1] for r in ranges], np.int32)
        P = int(np.prod([hi - lo + 1 for lo, hi in ranges]))
        val, fl = kc.col_wide(rng, m), kc.flags(rng, m, 0.4)
        ok = [np.zeros(P, np.int32) for _ in range(g)]
        osum, occ = np.zeros(P, np.uint64), np.zeros(P, np.uint32)
        L.ref_groupby_sum(R.ptr_array(keys), R.ptr(mins), R.ptr(maxs), g, R.ptr(val), R.ptr(fl), m, P,
                          R.ptr_array(ok), R.ptr(osum), R.ptr(occ))
        ins = {"val": val, "flags": fl, "mins": mins, "maxs": maxs}
        outs = {"sum": osum, "occ": (occ != 0).astype(np.uint8)}
        for j in range(g):
            ins["key%d" % j] = keys[j]
            outs["okey%d" % j] = np.where(occ != 0, ok[j], 0).astype(np.int32)
        add("groupby_%d" % g, "groupby", {"g": g, "P": P}, ins, outs)
    for nb in (1, 40, 1500):
        rng = np.random.default_rng(6000 + nb)
        lo = 1
        keys = kc.unique_keys(rng, nb, lo)
        bfl = kc.flags(rng, nb, 0.3)
        ht = np.zeros(nb, np.uint8)
        L.ref_ht_build_keys(R.ptr(keys), R.ptr(bfl), nb, R.ptr(ht), lo, nb)
        m = 5 * nb + 13
        probe = rng.integers(lo - 3, lo + nb + 3, m).astype(np.int32)
        fin = kc.flags(rng, m, 0.8)
        out = np.empty(m, np.uint8)
        L.ref_probe_semi(R.ptr(probe), R.ptr(fin), R.ptr(out), m, R.ptr(ht), lo, lo + nb - 1)
        add("semi_%d" % nb, "semi", {"lo": lo, "len": nb},
            {"keys": keys, "bflags": bfl, "probe": probe, "in": fin}, {"ht": ht, "out": out})
        vals = kc.col_wide(rng, nb)
        ht2 = np.zeros(2 * nb, np.int32)
        L.ref_ht_build_kv(R.ptr(keys), R.ptr(vals), R.ptr(bfl), nb, R.ptr(ht2), lo, nb)
        out2 = np.empty(m, np.uint8)
        vout = np.full(m, -7, np.int32)
        L.ref_probe_full(R.ptr(probe), R.ptr(vout), R.ptr(fin), R.ptr(out2), m, R.ptr(ht2), lo, lo + nb - 1)
        add("full_%d" % nb, "full", {"lo": lo, "len": nb},
            {"keys": keys, "vals": vals, "bflags": bfl, "probe": probe, "in": fin},
            {"ht2": ht2, "out": out2, "val_out": vout})
    for p in (0.0, 0.5):
        rng = np.random.default_rng(7000 + int(p * 10))
        fl = kc.flags(rng, 30011, p)
        c = np.array([L.ref_count_flags(R.ptr(fl), fl.size)], np.uint64)
        add("count_%d" % int(p * 10), "count", {}, {"flags": fl}, {"count": c})
    return cases, arrays


PLAN_CASES = [
    ("filter_sum_1993", 0.01, "filter_sum", {"year": 1993}),
    ("filter_sum_1997", 0.01, "filter_sum", {"year": 1997}),
    ("date_join_1994", 0.01, "date_join", {"year0": 1994}),
    ("star_r1_c1", 0.02, "star", {"region": 1, "category": 1}),
    ("star_r3_c17", 0.02, "star", {"region": 3, "category": 17}),
    ("star_batched_shape", 0.02, "star", {"region": 2, "category": 5, "year_lo": 1993, "year_hi": 1996,
                                          "brand_count": 9}),
]


def plan_of(kind, kw):
    return {"filter_sum": plans.plan_filter_sum, "date_join": plans.plan_date_join, "star": plans.plan_star}[kind](**kw)


def naive_of(kind, kw, ds):
    f = ds["lineorder"]
    if kind == "filter_sum":
        return naive.filter_sum(f, **kw)
    if kind == "date_join":
        return naive.date_join(f, ds["ddate"], **kw)
    return naive.star(f, ds["supplier"], ds["part"], ds["ddate"], **kw)


def plan_cases():
    out = []
    for name, sf, kind, kw in PLAN_CASES:
        ds = datasets.dataset(sf)
        plan = plan_of(kind, kw)
        rows = datasets.oracle_run(ds, plan)
        assert rows == naive_of(kind, kw, ds), name
        sums = {t: {str(c): datasets.checksum(a) for c, a in sorted(cols.items())} for t, cols in ds.items()}
        out.append({"name": name, "sf": sf, "seed": 20240601, "kind": kind, "args": kw, "plan": plan,
                    "rows": [list(r) for r in rows], "checksums": sums})
    return out


def main():
    cases, arrays = kernel_cases()
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **arrays)
    with open(os.path.join(HERE, "kernels.json"), "w") as f:
        json.dump(cases, f, indent=1)
    with open(os.path.join(HERE, "plans.json"), "w") as f:
        json.dump(plan_cases(), f, indent=1)
    print("wrote %d kernel cases, %d plan cases" % (len(cases), len(PLAN_CASES)))


if __name__ == "__main__":
    main()
