"""Benchmark: SSB-shaped three-way star join with group-by at SF20 on one GB300.

A step is one execution of the star-join plan (supplier semi join on region,
part join on category, date join; group by (d_year, p_brand1); SUM(lo_revenue))
over 120,000,000 seeded fact rows through the C-ABI executor, from plan text
to result rows in host memory.

  value      fact rows/s with the base columns resident in HBM (timed with
             CUDA events on the executor's stream over exactly K steps); the
             engine runs with its plan cache, so from the second execution on
             a step replays the prepared plan as one CUDA graph (every kernel
             runs every step; the host-side planning is reused).  The plain
             path's time per step is reported beside it
  e2e        the same metric with HOST (pinned) base columns: every step
             registers the tables (H2D copies, segment min/max) and executes
  roofline   the dominant kernel (the fused fact-side chain): algorithmic bytes
             (4 fact columns x 4 B x rows) / its CUDA-event duration, against
             the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (operator-at-a-time C/OpenMP restatement of
             the reference executor) on a bounded row sample, host cores
  batched    64 star-join plans over fact partitions of 1M..50M rows
             (lognormal), SF20 dimensions: queries/s and p50/p99 latency of the
             prepared batch (one CUDA graph, one persistent chain-batch launch)
             against the same 64 plans executed one at a time, results
             compared plan by plan
  served     SF50 fact (300M rows x 17 columns) resident; a seeded Poisson
             stream of mixed plans (filter-sum, date join, star join, star join
             with year/brand windows) replayed open-loop through the request
             server (continuous batching, 60 GB admission budget, shared
             scans: two plans' fact chains over the same rows in one paired
             pass) and through the plain one-at-a-time path: queries/s and
             p50/p99 latency per arrival rate, results compared request by
             request
  widened    the SSB flight-3 and flight-4 shapes at SF20 (rows/s, fused-pass
             roofline), device ORDER BY throughput and the columnar loader
             (--no-widened skips it)
  gpu_launches  kernels of the prepared plan's graph x steps

--unfused measures the operator-at-a-time path (one kernel per reference
operator) instead of the fused one.

--impl reference times the reference path's CPU restatement (the oracle port:
the reference itself needs AdaptiveCpp, oneDPL and Thrift and cannot be built
here) on the same metric.  Under torchrun (--gpus N > 1) each rank runs its
own fact partition (weak scaling, no collective on the data path); rank 0
prints the line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rows/s & %HBM roofline (SF20 star join); batched qps + p99 vs plain"
UNIT = "rows/s"
SF = 20.0
REGION, CATEGORY = 2, 11


def _plan_star():
    from sycldb_gb300 import plans

    return plans.plan_star(REGION, CATEGORY)


def _plan_filter_sum():
    from sycldb_gb300 import plans

    return plans.plan_filter_sum(1994)


def _plan_date_join():
    from sycldb_gb300 import plans

    return plans.plan_date_join(1994)


# name -> (plan builder, fact columns key, dominant kernel)
PLANS = {
    "star": (_plan_star, "star", "k_dense (fused chain: semi + full + full probe, warp compaction, group-by; the "
                                 "tuned variant, at SF20 the bound pass with late columns)"),
    "filter_sum": (_plan_filter_sum, "q1", "k_dense (fused chain: range + range + select + projection, sum)"),
    "date_join": (_plan_date_join, "q2", "k_dense (fused chain: range + full probe + projection, group-by)"),
}
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "fused_chain_star_sf20.txt")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--plan", default="star", choices=sorted(PLANS),
                    help="plan of the main measurement (the headline is the star join; the others profile the "
                         "filter-sum and date-join passes)")
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sf", type=float, default=SF)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the SF1 configurations (filter-project-sum, date join + group-by)")
    ap.add_argument("--only", default="", choices=["", "configs", "pairs"],
                    help="run one section alone (for profiling): configs")
    ap.add_argument("--config-names", default="",
                    help="comma-separated subset of the SF1 configurations to run (default: all)")
    ap.add_argument("--config-copies", type=int, default=8,
                    help="copies of the SF1 fact columns the configs section rotates through (L2 defeat)")
    ap.add_argument("--no-widened", action="store_true",
                    help="skip the widened rows (flight-3 / flight-4 shapes, device ORDER BY, columnar loader)")
    ap.add_argument("--unfused", action="store_true",
                    help="operator at a time: one kernel per reference operator (K1-K16), no fused chains; "
                         "the roofline is then over the step's summed kernel time")
    ap.add_argument("--e2e-steps", type=int, default=10, help="0 skips the host-buffer leg")
    ap.add_argument("--arena-gb", type=float, default=0.0, help="executor arena; 0 = the default budget")
    ap.add_argument("--batched-runs", type=int, default=20,
                    help="timed runs of the 64-plan batch (0 skips the batched form)")
    ap.add_argument("--plain-rounds", type=int, default=3, help="timed rounds of the 64 plans one at a time")
    ap.add_argument("--batched-plans", type=int, default=64, help="plans (fact partitions) in the batch")
    ap.add_argument("--batched-median", type=float, default=7e6,
                    help="median partition rows (lognormal, clipped to [1M, 50M]); smaller values make a small "
                         "case of the same kernel for profiling")
    ap.add_argument("--served-rates", default="50,200,500,1000,2000",
                    help="Poisson arrival rates (queries/s) of the served form; empty skips it")
    ap.add_argument("--served-seconds", type=float, default=1.5, help="arrival span per rate (at least 100 requests)")
    ap.add_argument("--served-slots", type=int, default=4, help="served form: batches in flight at once")
    ap.add_argument("--no-shared-scans", action="store_true",
                    help="served form: every fact chain on its own (no paired passes)")
    return ap.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "20"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.05)
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


CONFIG_PROFILES = {"filter_project_sum_sf1": os.path.join(ROOT, "profiles", "fused_chain_filter_sum_sf1.txt"),
                   "date_join_groupby_sf1": os.path.join(ROOT, "profiles", "fused_chain_date_join_sf1.txt")}


def profile_traffic(path=PROFILE_SUMMARY, key="traffic_bytes_per_launch_sf20:"):
    """DRAM bytes per launch of a fused chain from its committed ncu summary."""
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


def dims_host(sf):
    from sycldb_gb300 import ssb

    d = ssb.gen_dims(sf)
    return {t: d[t] for t in ("supplier", "part", "ddate")}


# ---------------------------------------------------------------------- CPU
# The CPU leg: the oracle (operator-at-a-time C/OpenMP restatement of the
# reference executor) over the same seeded inputs, generated by the oracle's
# own generator, so that this leg loads nothing of the native library.  It
# runs the whole workload (no sampling) with the step/warm-up counts of the
# GPU arm: W untimed repetitions, then K timed ones (the reference's own
# method is 10 repetitions with the first dropped, common.hpp:5,
# app/application.cpp:37-48).

CPU_CONFIGS = {
    # name -> (plan builder, fact column key, SF, dimensions read)
    "filter_project_sum_sf1": (_plan_filter_sum, "q1", 1.0, ()),
    "date_join_groupby_sf1": (_plan_date_join, "q2", 1.0, ("ddate",)),
}


def cpu_oracle_time(plan: dict, fact: dict, dims: dict, steps: int, warmup: int):
    """Times the oracle executor on one plan; returns (per-step seconds of the
    timed steps, canonical result rows, threads)."""
    from oracle import oracle as O

    tables = {"lineorder": O.make_table("lineorder", fact)}
    for t, cols in dims.items():
        tables[t] = O.make_table(t, cols)
    ex = O.OracleExecutor(tables)
    res = None
    for _ in range(warmup):
        res = ex.execute(plan)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        res = ex.execute(plan)
        times.append(time.perf_counter() - t0)
    return times, O.canonical_rows(res), O.lib().o_num_threads()


def cpu_workload(sf: float, cols, dim_names):
    """Seeded fact and dimension columns from the oracle's generator."""
    from oracle import build_oracle

    build_oracle.build_oracle()
    from oracle import oracle as O
    from sycldb_gb300 import ssb

    gen = O.OracleGen()
    fact = ssb.gen_lineorder_host(ssb.fact_rows(sf), cols, sf, gen=gen)
    dims = ssb.gen_dims(sf, gen=gen)
    return fact, {t: dims[t] for t in dim_names}


def _cpu_line(n: int, times, cores: int):
    mean = sum(times) / len(times)
    return {"value": n / mean, "unit": UNIT, "ms_per_step": mean * 1e3,
            "ms_median": statistics.median(times) * 1e3, "cores": cores, "kind": "port"}


def cpu_reference_all(sf: float, steps: int, warmup: int, configs: bool = True):
    """The headline star join at full size, then (configs) the SF1
    configurations; every result's canonical rows are returned with it."""
    from sycldb_gb300 import ssb

    n = ssb.fact_rows(sf)
    fact, dims = cpu_workload(sf, ssb.QUERY_COLUMNS["star"], ("supplier", "part", "ddate"))
    times, rows, cores = cpu_oracle_time(_plan_star(), fact, dims, steps, warmup)
    main = _cpu_line(n, times, cores)
    main["rows"] = rows
    del fact
    out = {}
    if configs:
        for name, (builder, key, csf, dnames) in CPU_CONFIGS.items():
            cn = ssb.fact_rows(csf)
            cfact, cdims = cpu_workload(csf, ssb.QUERY_COLUMNS[key], dnames)
            ct, crows, _ = cpu_oracle_time(builder(), cfact, cdims, steps, warmup)
            out[name] = _cpu_line(cn, ct, cores)
            out[name]["rows"] = crows
    return main, out


def run_reference(args, rank, world, pg):
    if rank != 0:
        return 0
    from sycldb_gb300 import ssb

    n = ssb.fact_rows(args.sf)
    main, cfgs = cpu_reference_all(args.sf, args.steps, args.warmup, configs=not args.no_configs)
    sample = ("the whole workload per step (%d fact rows, full dimensions): %d untimed repetitions, then %d "
              "timed; inputs from the oracle's own seeded generator" % (n, args.warmup, args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32/uint64", "data": DATA,
        "config": workload_config(args.sf, len(main["rows"])),
        "cpu_baseline": {"value": main["value"], "unit": UNIT, "cores": main["cores"], "kind": "port",
                         "sample": sample, "ms_median": main["ms_median"]},
        "e2e": {"value": main["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "configs": {k: {kk: vv for kk, vv in v.items() if kk != "rows"} for k, v in cfgs.items()},
        "result_digests": {"star": rows_digest(main["rows"]), **{k: rows_digest(v["rows"]) for k, v in cfgs.items()}},
        "note": "CPU restatement of the reference executor (oracle port: C/OpenMP kernels, operator at a "
                "time, all host threads); the reference's SYCL CPU path needs AdaptiveCpp, oneDPL and Thrift, "
                "absent here",
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline_child(args):
    """Runs the CPU leg in a child process (its own address space, before
    the GPU work) and returns its JSON line, or None."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", str(args.steps),
           "--warmup", str(max(1, args.warmup)), "--sf", str(args.sf)]
    if args.no_configs:
        cmd.append("--no-configs")
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1800)
    for line in r.stdout.splitlines():
        if line.startswith("{"):
            return json.loads(line)
    print("cpu baseline leg failed (rc %d): %s" % (r.returncode, r.stderr[-2000:]), file=sys.stderr)
    return None


DATA = "synthetic (seeded SplitMix64 columns, SSB SF20 shapes)"


def rows_digest(rows) -> str:
    """SHA-256 of canonical result rows (sorted tuples of ints): what the two
    arms compare."""
    import hashlib

    return hashlib.sha256(json.dumps([list(map(int, r)) for r in rows]).encode()).hexdigest()


def workload_config(sf, groups):
    """The workload part of the bench line's config, the same in both arms."""
    from sycldb_gb300 import ssb

    n = ssb.fact_rows(sf)
    return {"workload": workload_name(sf), "fact_rows_per_gpu": n, "groups": groups,
            "l2": "inputs larger than L2 (%.2f GB of fact columns per step)" % (16 * n / 1e9),
            "parallelism": "1 GPU"}


def workload_name(sf):
    return ("SSB-shaped star join SF%g: %d fact rows x (partkey, suppkey, orderdate, revenue); supplier %d, "
            "part %d, date 2556; s_region=%d semi join, p_category=%d, group by (d_year, p_brand1), "
            "SUM(lo_revenue)" % (sf, int(6e6 * sf), int(2000 * sf), int(54000 * sf), REGION, CATEGORY))


# ---------------------------------------------------------------------- GPU
def run_ours(args, rank, world, local, pg):
    import torch

    from sycldb_gb300 import build, capi, plans, ssb

    build.build()
    torch.cuda.set_device(local)
    from sycldb_gb300.engine import Engine

    # the CPU leg first, in a child process, before any device work
    ref = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.plan == "star":
        ref = cpu_baseline_child(args)
    if args.only == "configs":
        out = run_configs(args, rank, torch.cuda.Stream(), measured_peaks()[0], ref)
        if rank == 0:
            print(json.dumps({"configs": out}), flush=True)
        return 0
    if args.only == "pairs":
        out = run_pairs(args, args.sf)
        if rank == 0:
            print(json.dumps({"shared_scans": out}), flush=True)
        return 0

    L = capi.lib()
    sf = args.sf
    n = ssb.fact_rows(sf)
    build_plan, cols_key, kernel_name = PLANS[args.plan]
    cols = ssb.QUERY_COLUMNS[cols_key]
    # plan text, serialised once: what a caller of sdb_engine_execute holds
    plan = json.dumps(build_plan())
    dims = dims_host(sf)
    fact = ssb.gen_lineorder_device(n, cols, sf, salt=rank)
    torch.cuda.synchronize()

    stream = torch.cuda.Stream()
    arena = int(args.arena_gb * (1 << 30))

    # (1) the plain path with every launch timed by CUDA events: the fused
    # kernel's time per launch (roofline) and the launches of one execution
    fuse = not args.unfused
    peng = Engine(arena_bytes=arena, fuse=fuse, profile=True, stream=stream.cuda_stream)
    peng.load_table("lineorder", fact)
    for t, c in dims.items():
        peng.load_table(t, c)
    res = None
    for _ in range(max(3, args.warmup)):
        res = peng.execute(plan)
    n_groups = res.nrows
    prof_steps = max(1, min(args.steps, 50))
    torch.cuda.synchronize()
    launches0 = L.sdb_launch_count()
    fused_ms, fused_launches = 0.0, 0
    pev0, pev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pev0.record(stream)
    for _ in range(prof_steps):
        peng.execute(plan)
        st = peng.kernel_stats()
        if not fuse:  # the whole step's kernels
            fused_launches += 1
            fused_ms += sum(v[1] for v in st.values())
        elif "fused_chain" in st:
            fused_launches += st["fused_chain"][0]
            fused_ms += st["fused_chain"][1]
    pev1.record(stream)
    pev1.synchronize()
    launches_per_step = (L.sdb_launch_count() - launches0) / prof_steps
    plain_ms_per_step = pev0.elapsed_time(pev1) / prof_steps
    stats_last = peng.kernel_stats()
    peng.close()

    # (2) the headline: the same plan through the engine with its plan cache
    # (from the second execution on, the prepared plan replays as one CUDA
    # graph: every kernel runs each step, only host-side planning is reused)
    eng = Engine(arena_bytes=arena, fuse=fuse, plan_cache=4, stream=stream.cuda_stream)
    eng.load_table("lineorder", fact)
    for t, c in dims.items():
        eng.load_table(t, c)
    for _ in range(max(3, args.warmup)):
        res = eng.execute(plan)
    assert res.nrows == n_groups
    star_rows = res.canonical()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.1)
    barrier(pg)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        eng.execute(plan)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    # a step replays the prepared plan: a one-plan batch with only its builds
    # batched, whose kernels are counted when its graph is captured
    with eng.batch([plan], chain_batch="builds" if fuse else False) as pb:
        graph_launches = pb.stats()["kernels_per_run"]
    launches = int(graph_launches * args.steps)
    elapsed_ms = ev0.elapsed_time(ev1)
    elapsed_ms = max_over_ranks(pg, elapsed_ms)
    ms_per_step = elapsed_ms / args.steps
    total_rows = sum_over_ranks(pg, float(n)) * args.steps
    value = total_rows / (elapsed_ms / 1e3)

    # roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    alg_bytes = 4 * len(cols) * n
    per_launch_ms = fused_ms / max(1, fused_launches)
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9 if fused_launches else None
    traffic = profile_traffic() if (args.plan == "star" and sf == SF and fuse) else None
    roof = {"kernel": kernel_name if fuse else "operator-at-a-time step (every K1-K16 launch of one execution)",
            "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
            "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
            "dram_gbs": (traffic / per_launch_ms / 1e6) if (traffic and per_launch_ms) else None,
            "traffic_note": ("DRAM bytes per launch from the committed ncu summary; below the algorithmic bytes "
                             "when the pass reads late columns only in the sectors of the rows that reach them"
                             if traffic else None),
            "launch_ms": per_launch_ms, "launches": fused_launches,
            "timing": "CUDA events around each %s on the executor stream, %d plain-path steps" %
                      ("fused-pass launch" if fuse else "kernel launch, summed per step", prof_steps)}

    # e2e through the C ABI with host (pinned) buffers
    e2e = run_e2e(args, eng, plan, n, cols, sf, rank, stream, pg) if args.e2e_steps > 0 else None
    eng.close()
    del fact
    torch.cuda.empty_cache()
    configs = run_configs(args, rank, stream, peak, ref) if not args.no_configs else None
    batched = run_batched(args, rank, world, local, pg, stream, peak) if args.batched_runs > 0 else None
    served = run_served(args, rank, world, local, pg, stream) if args.served_rates.strip() else None
    widened = run_widened(args, rank, stream, peak) if not args.no_widened else None
    shared = run_pairs(args, sf) if not args.no_widened else None

    if args.plan == "star":
        config = workload_config(sf, n_groups)
        if world > 1:
            config["parallelism"] = "replicas"
    else:
        config = {"workload": "%s plan, SF%g (%d fact rows)" % (args.plan, sf, n), "fact_rows_per_gpu": n,
                  "groups": n_groups, "l2": "inputs larger than L2 (%.2f GB of fact columns per step)" %
                  (alg_bytes / 1e9), "parallelism": "replicas" if world > 1 else "1 GPU"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/uint64", "data": DATA,
        "config": config,
        "engine": {"segment_rows": 1 << 28, "fused": fuse,
                   "plan_cache": "on: steps 2.. replay the prepared plan as one CUDA graph (all kernels run)",
                   "plain_path_ms_per_step": plain_ms_per_step},
        "roofline": roof,
        "configs": configs,
        "e2e": e2e,
        "batched": batched,
        "served": served,
        "widened": widened,
        "shared_scans": shared,
        "gpu_launches": launches,
        "gpu_launches_note": "kernels of the prepared plan's graph (%d: the dimension builds in one launch, the "
                             "fused chain, the result compaction) x steps; the plain path launches %d per "
                             "execution" % (graph_launches, int(round(launches_per_step))),
        "kernel_ms_last_step": {k: v[1] for k, v in stats_last.items()},
        "clocks": clk,
    }
    if ref is not None:
        cb = dict(ref["cpu_baseline"])
        cb["bit_exact_vs_gpu"] = rows_digest(star_rows) == ref["result_digests"]["star"]
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_configs(args, rank, stream, peak, ref):
    """The SF1 configurations (6 M fact rows): filter-project-sum and filter +
    date join + group-by by year.  The fact columns (72-96 MB) would stay in
    the 126 MB L2 from one step to the next, so the section keeps
    ``--config-copies`` copies of them in separate buffers (768 MB for the
    filter-project-sum) and step i runs on copy i mod copies: every step
    reads its columns from HBM.  Per configuration: rows/s through the
    prepared plans (CUDA events over K steps), the fused kernel's time per
    launch from the plain path (CUDA events around each launch) and its
    roofline over the referenced fact columns, and the CPU leg's time and
    result on the same inputs."""
    import torch

    from sycldb_gb300 import ssb
    from sycldb_gb300.engine import Engine

    out = {}
    copies = max(1, args.config_copies)
    wanted = [x for x in args.config_names.split(",") if x]
    for name, (builder, key, csf, dnames) in CPU_CONFIGS.items():
        if wanted and name not in wanted:
            continue
        n = ssb.fact_rows(csf)
        cols = ssb.QUERY_COLUMNS[key]
        base = ssb.gen_lineorder_device(n, cols, csf, salt=rank)
        tabs = [{c: base[c].clone() for c in cols} for _ in range(copies)]
        del base
        dims = ssb.gen_dims(csf)
        pls = [json.dumps(_with_fact_tag(builder, i)) for i in range(copies)]
        torch.cuda.synchronize()

        def loaded(**kw):
            e = Engine(fuse=True, stream=stream.cuda_stream, **kw)
            for i, t in enumerate(tabs):
                e.load_table("lineorder@%d" % i, t)
            for d in dnames:
                e.load_table(d, dims[d])
            return e

        # the fused kernel's time per launch (plain path, every launch timed)
        peng = loaded(profile=True)
        for i in range(copies * 2):
            peng.execute(pls[i % copies])
        kms, kn, prof = 0.0, 0, max(copies * 3, min(args.steps, 64))
        for i in range(prof):
            peng.execute(pls[i % copies])
            st = peng.kernel_stats()
            if "fused_chain" in st:
                kn += st["fused_chain"][0]
                kms += st["fused_chain"][1]
        peng.close()
        # rows/s through the prepared plans
        eng = loaded(plan_cache=copies + 2)
        rows = None
        for _ in range(max(3, args.warmup)):
            for p in pls:
                rows = eng.execute(p).canonical()
        exact_copies = all(eng.execute(p).canonical() == rows for p in pls)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            eng.execute(pls[i % copies])
        e1.record(stream)
        e1.synchronize()
        eng.close()
        ms = e0.elapsed_time(e1) / args.steps
        alg = 4 * len(cols) * n
        per = kms / max(1, kn)
        ach = alg / (per / 1e3) / 1e9 if kn else None
        entry = {
            "workload": "%s: %d fact rows x %d int32 columns (%s)" % (name, n, len(cols), ", ".join(
                "lo_col%d" % c for c in cols)),
            "rows_per_s": n / (ms / 1e3), "ms_per_step": ms, "steps": args.steps, "groups": len(rows),
            "l2": "%d copies of the fact columns (%.0f MB), step i reads copy i mod %d: inputs not L2-resident "
                  "between steps" % (copies, copies * alg / 1e6, copies),
            "roofline": {"kernel": "k_dense (fused chain)", "bound": "hbm", "achieved": ach, "peak": peak,
                         "unit": "GB/s", "frac": (ach / peak) if ach else None, "launch_ms": per,
                         "launches": kn, "algorithmic_bytes_per_launch": alg,
                         "traffic": profile_traffic(CONFIG_PROFILES[name], "traffic_bytes_per_launch:"),
                         "timing": "CUDA events around each fused-pass launch, %d plain-path steps" % prof},
            "same_rows_every_copy": exact_copies,
        }
        if ref is not None and name in (ref.get("configs") or {}):
            cb = dict(ref["configs"][name])
            cb["sample"] = "the whole workload, %d untimed + %d timed repetitions" % (max(1, args.warmup),
                                                                                       args.steps)
            cb["bit_exact_vs_gpu"] = rows_digest(rows) == ref["result_digests"][name]
            entry["cpu_baseline"] = cb
        out[name] = entry
        del tabs
        torch.cuda.empty_cache()
    return out


def _with_fact_tag(builder, tag):
    """The configuration's plan over fact table lineorder@tag."""
    from sycldb_gb300 import plans

    p = builder()
    for r in p["rels"]:
        if r.get("relOp") == "TABLE_SCAN" and r["tables"][-1] == "lineorder":
            r["tables"] = list(r["tables"][:-1]) + ["lineorder@%d" % tag]
    return p


def run_e2e(args, eng, plan, n, cols, sf, rank, stream, pg):
    import torch

    from sycldb_gb300 import ssb

    pinned = {c: torch.empty(n, dtype=torch.int32, pin_memory=True) for c in cols}
    host = ssb.gen_lineorder_host(n, cols, sf, salt=rank, out={c: t.numpy() for c, t in pinned.items()})
    dims = {}
    for t, dcols in dims_host(sf).items():  # dimension columns pinned too
        dims[t] = {}
        for c, a in dcols.items():
            pt = torch.empty(a.size, dtype=torch.int32, pin_memory=True)
            pt.numpy()[:] = a
            dims[t][c] = pt.numpy()
    h2d = sum(a.nbytes for a in host.values()) + sum(a.nbytes for d in dims.values() for a in d.values())

    # the host-to-device link alone: best of 3 copies of one pinned column
    probe_src = pinned[cols[0]]
    probe_dst = torch.empty_like(probe_src, device="cuda")
    link = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        probe_dst.copy_(probe_src, non_blocking=True)
        torch.cuda.synchronize()
        link.append(probe_src.numel() * 4 / (time.perf_counter() - t0) / 1e9)
    del probe_dst
    h2d_gbs = max(link)

    def step():
        eng.load_table("lineorder", host)
        for t, c in dims.items():
            eng.load_table(t, c)
        return eng.execute(plan)

    for _ in range(2):
        r = step()
    d2h = sum(c.nbytes for c in r.columns)
    torch.cuda.synchronize()
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        step()
    torch.cuda.synchronize()
    dt = max_over_ranks(pg, time.perf_counter() - t0)
    rows = sum_over_ranks(pg, float(n)) * args.e2e_steps
    ms = dt / args.e2e_steps * 1e3
    floor_ms = h2d / (h2d_gbs * 1e9) * 1e3
    return {"value": rows / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": ms, "steps": args.e2e_steps,
            "timing": "host wall clock around load_table(host pinned columns) + execute, synchronised",
            "link_bound": {"h2d_gbs": h2d_gbs, "floor_ms": floor_ms, "frac": floor_ms / ms,
                           "note": "the step's host-to-device bytes at the measured pinned copy bandwidth; "
                                   "more streams or copy engines do not raise it on this box"}}


def _pct(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
    return xs[k]


def run_pairs(args, sf, reps=15):
    """Shared scans: for each served shape (star join, date join,
    filter-project-sum), a batch of two plans with their own literals over
    one fact table (builds batched, fact chains on their own), run with the
    paired pass and with each chain on its own: device ms per run (median),
    results compared plan by plan."""
    import numpy as np
    import torch

    from sycldb_gb300 import plans, ssb
    from sycldb_gb300.engine import Engine

    n = ssb.fact_rows(sf)
    fact = ssb.gen_lineorder_device(n, (3, 4, 5, 8, 9, 11, 12), sf, salt=0)
    dims = dims_host(sf)
    torch.cuda.synchronize()
    kinds = {
        "star_join": [plans.plan_star(1, 3), plans.plan_star(2, 11)],
        "date_join": [plans.plan_date_join(1995), plans.plan_date_join(1997)],
        "filter_project_sum": [plans.plan_filter_sum(1994, 1, 3, 25), plans.plan_filter_sum(1993, 4, 6, 35)],
    }
    out = {}
    for shared in (True, False):
        with Engine(shared_scans=shared) as eng:
            eng.load_table("lineorder", fact)
            for t, c in dims.items():
                eng.load_table(t, c)
            for k, pls in kinds.items():
                pls = [json.dumps(p) for p in pls]
                alone = [eng.execute(p).canonical() for p in pls]
                with eng.batch(pls, chain_batch="builds") as b:
                    for _ in range(3):
                        b.run()
                    ms = []
                    for _ in range(reps):
                        got = [r.canonical() for r in b.run()]
                        assert got == alone, k
                        ms.append(b.stats()["last_run_ms"])
                    st = b.stats()
                e = out.setdefault(k, {})
                e["paired_ms" if shared else "apart_ms"] = float(np.median(ms))
                if shared:
                    e["paired_chains"] = st["paired_chains"]
    for e in out.values():
        e["speedup"] = e["apart_ms"] / e["paired_ms"]
    del fact
    torch.cuda.empty_cache()
    return {"workload": "SF%g lineorder (%d rows); per shape a batch of two plans with their own literals, "
                        "dimension builds in one launch, each fact chain on its own (apart) or both in one "
                        "paired pass; device ms per run, median of %d" % (sf, n, reps),
            "results": "each plan's rows equal its rows alone", "shapes": out}


def run_widened(args, rank, stream, peak):
    """The rows beyond the headline shape, measured the same way: the SSB
    flight-3 (three joins, three group-by keys) and flight-4 (four joins,
    revenue - supplycost) shapes at SF20 -- rows/s through the prepared plan
    and the fused kernel's roofline over its fact columns --, ORDER BY on the
    device (sdb_sort_rows throughput) and the columnar file loader."""
    import shutil
    import tempfile

    import numpy as np
    import torch

    from sycldb_gb300 import capi, plans, ssb
    from sycldb_gb300.engine import Engine

    out = {}
    sf = SF
    n = ssb.fact_rows(sf)
    dims = ssb.gen_dims(sf)
    shapes = {
        "flight3_customer_supplier_date": (plans.plan_customer_supplier_date(2), (2, 4, 5, 12)),
        "flight4_profit": (plans.plan_profit(1), (2, 3, 4, 5, 12, 13)),
    }
    fact = ssb.gen_lineorder_device(n, sorted({c for _, cs in shapes.values() for c in cs}), sf, salt=rank)
    torch.cuda.synchronize()

    def loaded(**kw):
        e = Engine(fuse=True, stream=stream.cuda_stream, **kw)
        e.load_table("lineorder", fact)
        for t, c in dims.items():
            e.load_table(t, c)
        return e

    for name, (plan, cs) in shapes.items():
        plan = json.dumps(plan)
        peng = loaded(profile=True)
        for _ in range(3):
            res = peng.execute(plan)
        kms, kn, prof_steps = 0.0, 0, 10
        for _ in range(prof_steps):
            peng.execute(plan)
            st = peng.kernel_stats()
            if "fused_chain" in st:
                kn += st["fused_chain"][0]
                kms += st["fused_chain"][1]
        peng.close()
        eng = loaded(plan_cache=4)
        for _ in range(3):
            eng.execute(plan)
        steps = 20
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            eng.execute(plan)
        e1.record(stream)
        e1.synchronize()
        eng.close()
        ms = e0.elapsed_time(e1) / steps
        per = kms / prof_steps  # fused-pass time of one execution
        alg = 4 * len(cs) * n
        out[name] = {"rows_per_s": n / (ms / 1e3), "ms_per_step": ms, "groups": res.nrows,
                     "fact_columns": list(cs), "fused_ms_per_execution": per,
                     "fused_launches_per_execution": kn / prof_steps,
                     "roofline_frac": (alg / (per / 1e3) / 1e9 / peak) if kn else None,
                     "note": "prepared plan, CUDA events over %d steps; roofline: %d B per fact row (every "
                             "referenced fact column once) over the fused passes' time per execution" %
                             (steps, 4 * len(cs))}
    del fact
    torch.cuda.empty_cache()

    # ORDER BY: a stable radix sort of row ids by (int32 asc, uint64 desc)
    m = 1 << 24
    g = torch.Generator(device="cuda").manual_seed(7)
    k0 = torch.randint(-2**31, 2**31 - 1, (m,), dtype=torch.int32, device="cuda", generator=g)
    k1 = torch.randint(0, 2**62, (m,), dtype=torch.int64, device="cuda", generator=g)
    perm = torch.empty(m, dtype=torch.int32, device="cuda")
    L = capi.lib()
    sb = L.sdb_sort_scratch_bytes(m)
    scratch = torch.empty(sb + 256, dtype=torch.uint8, device="cuda")
    sp = (scratch.data_ptr() + 255) // 256 * 256
    keys = (ctypes.c_void_p * 2)(k0.data_ptr(), k1.data_ptr())
    types = (ctypes.c_int * 2)(0, 1)
    desc = (ctypes.c_int * 2)(0, 1)
    for _ in range(2):
        capi.check(L.sdb_sort_rows(keys, types, desc, 2, m, perm.data_ptr(), sp, sb, stream.cuda_stream))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(5):
        capi.check(L.sdb_sort_rows(keys, types, desc, 2, m, perm.data_ptr(), sp, sb, stream.cuda_stream))
    e1.record(stream)
    e1.synchronize()
    sms = e0.elapsed_time(e1) / 5
    out["order_by_sort"] = {"rows": m, "keys": "int32 ascending, uint64 descending (12 passes of 8 bits)",
                            "ms": sms, "rows_per_s": m / (sms / 1e3)}
    del k0, k1, perm, scratch

    # the columnar loader: the reference's file layout, just written (so in
    # the page cache), read into device columns with min/max
    lsf = 2.0
    ln = ssb.fact_rows(lsf)
    lcols = ssb.QUERY_COLUMNS["star"]
    d = tempfile.mkdtemp(prefix="sdb_cols_")
    try:
        ssb.write_columnar(d, {"lineorder": ssb.gen_lineorder_host(ln, lcols, lsf)})
        with Engine(fuse=True, stream=stream.cuda_stream) as eng:
            times = []
            for _ in range(3):
                t0 = time.perf_counter()
                eng.load_dir(d, "lineorder", columns=list(lcols), background=False)
                torch.cuda.synchronize()
                times.append(time.perf_counter() - t0)
        best = min(times)
        nbytes = 4 * len(lcols) * ln
        out["load_dir"] = {"bytes": nbytes, "s": best, "gbs": nbytes / best / 1e9,
                           "note": "%d lineorder columns of %d rows from files in the page cache, 8 MB chunks "
                                   "read by 4 threads (two pinned buffers each), min/max on the device; "
                                   "best of 3" %
                                   (len(lcols), ln)}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return out


def run_batched(args, rank, world, local, pg, stream, peak):
    """The batched form against the plain one-plan-at-a-time path, same
    plans, same engine, same device-resident partitions."""
    import torch

    from sycldb_gb300 import ssb, workloads
    from sycldb_gb300.engine import Engine

    wl = workloads.batch_workload(n_plans=args.batched_plans, median=args.batched_median, seed=ssb.SEED + rank)
    eng = Engine(arena_bytes=int(args.arena_gb * (1 << 30)), fuse=True, stream=stream.cuda_stream)
    workloads.load_batch_tables(eng, wl, device=True)
    pls = wl.plans()
    torch.cuda.synchronize()

    alone = None
    for _ in range(2):
        alone = [eng.execute(p).canonical() for p in pls]
    lat_plain = []
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.plain_rounds):
        for p in pls:
            t = time.perf_counter()
            eng.execute(p)
            lat_plain.append(time.perf_counter() - t)
    plain_s = max_over_ranks(pg, time.perf_counter() - t0)

    b = eng.batch(pls)
    got = [r.canonical() for r in b.run()]
    exact = got == alone
    for _ in range(3):
        b.run()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.1)
    lat_b, dev_ms, chain_ms, pre_ms, post_ms, build_ms = [], [], [], [], [], []
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.batched_runs):
        t = time.perf_counter()
        b.run()
        lat_b.append(time.perf_counter() - t)
        st = b.stats()
        dev_ms.append(st["last_run_ms"])
        chain_ms.append(st["last_chain_ms"])
        pre_ms.append(st["last_pre_ms"])
        post_ms.append(st["last_post_ms"])
        build_ms.append(st["last_build_ms"])
    batch_s = max_over_ranks(pg, sum(lat_b))
    clk = clocks.stop()
    # the same runs without the Python conversion of the results, and without
    # unpacking at all: where the host time of a run goes
    lat_native, lat_bare = [], []
    for _ in range(max(3, args.batched_runs // 2)):
        t = time.perf_counter()
        b.run_native()
        lat_native.append(time.perf_counter() - t)
        t = time.perf_counter()
        b.run(unpack=False)
        lat_bare.append(time.perf_counter() - t)
    st = b.stats()
    b.close()
    eng.close()

    nq = len(pls)
    qps_plain = sum_over_ranks(pg, float(nq * args.plain_rounds)) / plain_s
    qps_batched = sum_over_ranks(pg, float(nq * args.batched_runs)) / batch_s
    chain_med = statistics.median(chain_ms)
    # the chain batch holds the fact chains of partitions under 2^23 rows
    # (larger ones run the single-chain kernel on their own)
    solo_rows = 1 << 23
    batched_rows = sum(r for r in wl.rows if r < solo_rows)
    fact_bytes = 16 * batched_rows
    achieved = fact_bytes / (chain_med / 1e3) / 1e9 if chain_med > 0 and fact_bytes else None
    dev_med = statistics.median(dev_ms)
    all_bytes = wl.algorithmic_bytes()
    return {
        "workload": "%d star-join plans (supplier region semi join, part category + brand window, date year "
                    "window; group by (d_year, p_brand1), SUM(lo_revenue)), each over its own fact partition; "
                    "partition rows lognormal (median %g, log-sd 1) clipped to [1M, 50M], total %d rows; SF20 "
                    "dimensions" % (nq, args.batched_median, wl.total_rows),
        "partition_rows": {"min": min(wl.rows), "max": max(wl.rows), "total": wl.total_rows},
        "group_counts": {"min": min(len(r) for r in alone), "max": max(len(r) for r in alone)},
        "qps_batched": qps_batched, "qps_plain": qps_plain, "speedup": qps_batched / qps_plain,
        "latency_ms": {
            "batched_p50": _pct(lat_b, 50) * 1e3, "batched_p99": _pct(lat_b, 99) * 1e3,
            "plain_p50": _pct(lat_plain, 50) * 1e3, "plain_p99": _pct(lat_plain, 99) * 1e3,
            "batched_p50_native_results": _pct(lat_native, 50) * 1e3,
            "batched_p50_no_unpack": _pct(lat_bare, 50) * 1e3,
            "note": "batched: every plan of a batch completes when the batch run returns (host wall clock "
                    "around sdb_batch_run incl. result unpacking); plain: each sdb_engine_execute alone"},
        "device_ms_per_batch": dev_med,
        "device_roofline": {"algorithmic_bytes": all_bytes, "achieved": all_bytes / (dev_med / 1e3) / 1e9,
                            "peak": peak, "unit": "GB/s", "frac": all_bytes / (dev_med / 1e3) / 1e9 / peak,
                            "note": "every referenced fact and dimension column read once, over the whole "
                                    "batch's device time"},
        "device_ms_phases": {"before_chains": statistics.median(pre_ms),
                             "builds": statistics.median(build_ms), "chains": statistics.median(chain_ms),
                             "after_chains": statistics.median(post_ms),
                             "note": "before_chains: zeroing, then on 16 streams the plans' own work, incl. "
                                     "the fact chains of partitions of 2^23 rows or more (single-chain "
                                     "kernel); builds: every dimension filter + hash-table build of the batch "
                                     "in one launch; chains: the chain batch (fact chains of smaller "
                                     "partitions); after_chains: compaction, gathers, result copy"},
        "chain_batch": {"kernel": "k_batch (persistent, span work queue; semi + full + full probe, group-by)",
                        "chains": sum(1 for r in wl.rows if r < solo_rows), "rows": batched_rows,
                        "ms": chain_med, "algorithmic_bytes": fact_bytes,
                        "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak if achieved else None},
        "kernels_per_run": st["kernels_per_run"], "graph": bool(st["graph"]),
        "chain_launches": st["chain_launches"], "batched_chains": st["batched_chains"],
        "batched_builds": st["batched_builds"],
        "arena_bytes": st["arena_bytes"], "bit_exact_vs_plain": exact,
        "plain_rounds": args.plain_rounds, "batched_runs": args.batched_runs, "clocks": clk,
    }


def run_served(args, rank, world, local, pg, stream):
    """The served form against the plain path on the same arrival traces."""
    import torch

    from sycldb_gb300 import ssb, workloads
    from sycldb_gb300.engine import Engine, Server, replay_plain

    sf = 50.0
    n = ssb.fact_rows(sf)
    eng = Engine(fuse=True, stream=stream.cuda_stream, shared_scans=not args.no_shared_scans)
    fact = ssb.gen_lineorder_device(n, range(17), sf, salt=rank)
    eng.load_table("lineorder", fact)
    for t, c in dims_host(sf).items():
        eng.load_table(t, c)
    torch.cuda.synchronize()
    rates = [float(x) for x in args.served_rates.split(",") if x.strip()]
    out = []
    clocks = ClockSampler(local)
    clocks.start()
    for rate in rates:
        nreq = max(100, int(rate * args.served_seconds))
        reqs = workloads.poisson_stream(rate, nreq, seed=ssb.SEED + rank)
        pls = [r.plan for r in reqs]
        at = [r.t for r in reqs]
        # warm both paths on requests of every plan kind (alone, then as one
        # burst), so that no kernel is loaded for the first time while timed
        warm = workloads.poisson_stream(1000.0, 32, seed=ssb.SEED + 99 + rank)
        wk = {}
        for r in warm:
            wk.setdefault(r.kind, []).append(r.plan)
        wpl = [p for ps in wk.values() for p in ps[:2]] + [r.plan for r in warm]
        replay_plain(eng, wpl, [0.0] * len(wpl), keep_results=False)
        pst, plat, pres, pwall = replay_plain(eng, pls, at)
        with Server(eng, budget_bytes=60 << 30, slots=args.served_slots) as srv:
            for p in wpl[:8]:
                srv.replay([p], [0.0], keep_results=False)
            srv.replay(wpl, [0.0] * len(wpl), keep_results=False)
            st0 = srv.stats()
            sst, slat, sres, swall = srv.replay(pls, at)
            st = srv.stats()
        ok = all(x == 0 for x in pst) and all(x == 0 for x in sst)
        exact = ok and all(a.canonical() == b.canonical() for a, b in zip(pres, sres))
        out.append({
            "rate_qps": rate, "requests": nreq,
            "served": {"qps": nreq / swall, "p50_ms": _pct(slat, 50), "p99_ms": _pct(slat, 99),
                       "batches": st["batches"] - st0["batches"],
                       "mean_batch": (st["batched_plans"] - st0["batched_plans"]) / max(1, st["batches"] - st0["batches"]),
                       "max_inflight_plans": st["max_inflight_plans"], "peak_device_bytes": st["peak_device_bytes"],
                       "paired_chains": st["paired_chains"] - st0["paired_chains"],
                       "dispatcher_ms_per_request": {
                           "sizing": (st["sizing_us"] - st0["sizing_us"]) / 1e3 / max(1, nreq),
                           "record_and_enqueue": (st["launch_us"] - st0["launch_us"]) / 1e3 / max(1, nreq)}},
            "plain": {"qps": nreq / pwall, "p50_ms": _pct(plat, 50), "p99_ms": _pct(plat, 99)},
            "bit_exact": exact,
        })
    clk = clocks.stop()
    eng.close()
    del fact
    torch.cuda.empty_cache()
    return {"workload": "SF50 lineorder resident (%d rows x 17 int32 columns), SF50 dimensions; Poisson arrivals, "
                        "plan mix 1/4 each: filter-project-sum (one-year window, discount range, quantity bound), "
                        "filter + date join + group by year, star join, star join with year and brand windows" % n,
            "latency": "host wall clock from each request's scheduled arrival to its result on the host",
            "budget_bytes": 60 << 30, "slots": args.served_slots, "rates": out, "clocks": clk,
            "shared_scans": "off" if args.no_shared_scans else
            "on: two fact chains of one shape over the same rows run as one paired pass (paired_chains)"}


def main():
    args = parse_args()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        rc = run_reference(args, rank, world, pg)
    else:
        rc = run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
