"""The oracle against the committed golden vectors (produced by the reference's
own kernel functors) and the committed plan results.  CPU only; runs on any
machine, with or without the reference checkout."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import datasets

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = json.load(open(os.path.join(HERE, "kernels.json")))
ARR = np.load(os.path.join(HERE, "kernels.npz"))
PLANS = json.load(open(os.path.join(HERE, "plans.json")))


def inputs(case):
    return {k: ARR["%s/in/%s" % (case["name"], k)].copy() for k in case["inputs"]}


def outputs(case):
    return {k: ARR["%s/out/%s" % (case["name"], k)] for k in case["outputs"]}


def run_oracle(case):
    """Runs the oracle kernel of a golden case; returns its outputs."""
    k, p, i = case["kernel"], case["params"], inputs(case)
    if k == "select_lit":
        out = np.empty(i["col"].size, np.uint8)
        O.select_lit(i["col"], p["v"], p["cmp"], p["logic"], i["in"], out)
        return {"out": out}
    if k == "select_cols":
        out = np.empty(i["a"].size, np.uint8)
        O.select_cols(i["a"], i["b"], p["cmp"], p["logic"], i["in"], out)
        return {"out": out}
    if k == "logical":
        out = np.empty(i["in"].size, np.uint8)
        O.logical(p["logic"], i["in"], i["local"], out)
        return {"out": out}
    if k == "fill_i32":
        out = np.zeros(outputs(case)["out"].size, np.int32)
        O.fill_i32(out, p["v"])
        return {"out": out}
    if k.startswith("binop_"):
        res = i["res0"].copy()
        mode = k.split("_")[1]
        if mode == "cc":
            O.binop_cc(res, i["a"], i["b"], p["op"], i["flags"])
        elif mode == "lc":
            O.binop_lc(res, p["la"], i["b"], p["op"], i["flags"])
        else:
            O.binop_cl(res, i["a"], p["lb"], p["op"], i["flags"])
        return {"res": res}
    if k == "sum":
        acc = np.array([p["acc0"]], np.uint64)
        O.sum_i32_u64(i["col"], i["flags"], acc)
        return {"acc": acc}
    if k == "groupby":
        g, P = p["g"], p["P"]
        keys = [i["key%d" % j] for j in range(g)]
        ok = [np.zeros(P, np.int32) for _ in range(g)]
        s, occ = np.zeros(P, np.uint64), np.zeros(P, np.uint32)
        O.groupby_sum(keys, i["mins"], i["maxs"], i["val"], i["flags"], P, ok, s, occ)
        out = {"sum": s, "occ": (occ != 0).astype(np.uint8)}
        for j in range(g):
            out["okey%d" % j] = np.where(occ != 0, ok[j], 0).astype(np.int32)
        return out
    if k == "semi":
        ht = np.zeros(p["len"], np.uint8)
        O.ht_build_keys(i["keys"], i["bflags"], ht, p["lo"], p["len"])
        out = np.empty(i["probe"].size, np.uint8)
        O.probe_semi(i["probe"], i["in"], out, ht, p["lo"], p["lo"] + p["len"] - 1)
        return {"ht": ht, "out": out}
    if k == "full":
        ht2 = np.zeros(2 * p["len"], np.int32)
        O.ht_build_kv(i["keys"], i["vals"], i["bflags"], ht2, p["lo"], p["len"])
        out = np.empty(i["probe"].size, np.uint8)
        vout = np.full(i["probe"].size, -7, np.int32)
        O.probe_full(i["probe"], vout, i["in"], out, ht2, p["lo"], p["lo"] + p["len"] - 1)
        return {"ht2": ht2, "out": out, "val_out": vout}
    if k == "count":
        return {"count": np.array([O.count_flags(i["flags"])], np.uint64)}
    raise KeyError(k)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_golden(case):
    got = run_oracle(case)
    for k, want in outputs(case).items():
        assert np.array_equal(got[k], want), (case["name"], k)


@pytest.mark.parametrize("case", PLANS, ids=[c["name"] for c in PLANS])
def test_oracle_plans_match_golden(case):
    ds = datasets.dataset(case["sf"], case["seed"])
    for t, sums in case["checksums"].items():
        for c, v in sums.items():
            assert datasets.checksum(ds[t][int(c)]) == v, "generator drift in %s%s" % (t, c)
    rows = datasets.oracle_run(ds, case["plan"])
    assert [list(r) for r in rows] == case["rows"]
