"""Benchmark: batched GPU RRT-Connect (solved queries/s) on 1024 Panda queries.

One step = solving one batch of queries (default: 1024 seeded Panda
narrow-passage shelf queries with the reference's shelf settings:
granularity 128, balance 2, tree_ratio 1, dynamic domain on).  Prints one
JSON line (the contract this repository's driver reads):

  value      solved queries/s of the batched persistent kernel, inputs resident
             in HBM, timed with CUDA events on the launching stream, L2
             flushed between steps
  e2e        the same through the C ABI, prrtc_solve_batch, on host buffers
             (the prrtc_query array a C or C++ caller passes; upload, solve
             and download of results and paths inside the timed call);
             e2e_python: the same through the Python wrapper, marshalling
             and unpacking included
  plain      the drop-in single-query form (prrtc_solve) on a sample of the
             same queries, one at a time
  roofline   the planner kernel's algorithmic FP32 FLOPs (counted in-kernel:
             canonical FK + the reference checker's executed tests x weights)
             per launch / launch time, against the device's measured FP32 FMA
             peak (neither the HBM nor the tensor roof applies: the validator
             is SIMT FP32 work on L1/L2-resident data)
  cpu_baseline  the CPU restatement of pRRTC's algorithm (oracle, all host
             threads) on a bounded sample of the same queries

`--impl reference` times that CPU restatement alone: the reference's planner
is not run on the GPU (its kernel writes tree nodes past max_samples and
path entries past its fixed path array without bounds checks), so its
algorithm restated on the CPU is the reference arm.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from prrtc_gb300.workloads import SETTINGS as WORKLOAD_SETTINGS  # noqa: E402

MARGIN = 1e-5   # planning margin (m): every returned path clears contact by 10 micrometres
GPU_BUDGET_NS = int(30e9)   # per batch launch; unsolved queries past it count as failures
CPU_BUDGET_S = 20.0         # per query in the CPU restatement


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.rows, self.proc = device, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(self.rows[0][1]) if self.rows[0][1].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(self.rows)}


def settings_for(name):
    from prrtc_gb300 import Settings
    return Settings(**WORKLOAD_SETTINGS[name])


def oracle_lib():
    sys.path.insert(0, str(ROOT / "oracle"))
    from pyoracle import OracleLib, build
    build()
    return OracleLib()


def cpu_planner(robot, qs, settings, threads):
    """pRRTC's algorithm restated on the CPU (oracle), OpenMP over queries."""
    O = oracle_lib()
    t = time.perf_counter()
    res, _ = O.solve_many(robot, np.stack([q.start for q in qs]), np.stack([q.goal for q in qs]),
                          [q.env for q in qs], settings, threads=threads, path_cap=16, budget_s=CPU_BUDGET_S)
    dt = time.perf_counter() - t
    return sum(r.solved for r in res), dt, res


def cpu_sample_size(name):
    return {"panda_tabletop": 256, "panda_shelf": 64, "fetch_mixed": 64, "baxter_mixed": 32}[name]


def reference_arm(args, rank, world):
    if rank != 0:
        return
    from prrtc_gb300 import workloads
    robot = workloads.WORKLOADS[args.workload][0]
    qs = workloads.make(args.workload, args.queries)
    ns = min(cpu_sample_size(args.workload), len(qs))
    threads = os.cpu_count() or 1
    s = settings_for(args.workload)
    for _ in range(args.warmup):
        cpu_planner(robot, qs[:max(1, ns // 8)], s, threads)
    tot_solved, tot_dt = 0, 0.0
    for k in range(args.steps):
        sample = qs[(k * ns) % len(qs):][:ns]
        solved, dt, _ = cpu_planner(robot, sample, s, threads)
        tot_solved += solved
        tot_dt += dt
    v = tot_solved / tot_dt
    line = {"impl": "reference", "metric": metric_name(args), "value": v, "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(args),
            "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{ns} of the {len(qs)} queries per step"},
            "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def metric_name(args):
    return f"solved queries/s, batched, {args.workload} ({args.queries} queries per step; 1 GB300, 100% revalidated)"


def config_of(args):
    from prrtc_gb300 import autotune, workloads
    return {"workload": f"{args.workload}_{args.queries}", "queries_per_step": args.queries,
            "steps_streamed": "the K steps' queries (distinct seeds) flow through one persistent launch with "
                              f"{args.queries} resident slots; queries are admitted as others finish",
            "settings": WORKLOAD_SETTINGS[args.workload], "planning_margin_m": MARGIN,
            "batch_shape": autotune.load(workloads.WORKLOADS[args.workload][0], args.workload),
            "l2": "flushed before the timed launch; each step's queries use fresh arena slots and scenes "
                  "(stream input > L2)", "parallelism": "queries sharded over ranks"}


def shard_seed0(rank: int, n: int, steps: int) -> int:
    """First query seed of a rank: ranks plan disjoint query sets (weak scaling)."""
    return rank * n * steps


def allreduce(maxes, sums, world: int, device: str = "cpu"):
    """Whole-job figures over ranks: elementwise maxima (times) and sums
    (counts, bytes).  Queries shard with no exchange on the data path; these
    figures are the only collective."""
    if world <= 1:
        return list(maxes), list(sums)
    import torch
    import torch.distributed as dist
    m = torch.tensor([float(v) for v in maxes] or [0.0], dtype=torch.float64, device=device)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(v) for v in sums] or [0.0], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return m.tolist()[:len(maxes)], c.tolist()[:len(sums)]


def reduce_over_ranks(t_dev: float, solved: int, world: int, device: str = "cpu"):
    """The slowest rank's device time and the total of solved queries."""
    (t,), (c,) = allreduce([t_dev], [solved], world, device)
    return t, int(c)


def bulk_and_tail(results):
    """The launch's bulk rate and its tail.  bulk: solved queries that
    finished by the 99th-percentile finish time, over that time (device
    clock from the launch's start), so one hard query's solve time does not
    set it.  tail: the query that ended the launch (solve and finish times,
    samples drawn, tree sizes, status), and every unsolved query's status,
    samples and tree sizes."""
    fin = np.array([r.finish_ns for r in results if r.solved], np.float64)
    if not len(fin):
        return None, None
    t99 = float(np.percentile(fin, 99))
    bulk = {"queries_per_s": float((fin <= t99).sum()) / (t99 * 1e-9), "p99_finish_ms": t99 / 1e6,
            "last_finish_ms": float(fin.max()) / 1e6}
    last = max(range(len(results)), key=lambda i: results[i].finish_ns)
    r = results[last]

    def desc(i, r):
        return {"query": i, "solved": bool(r.solved), "status": int(r.status), "solve_ms": r.kernel_ns / 1e6,
                "finish_ms": r.finish_ns / 1e6, "samples": int(r.samples), "start_tree_size": r.start_tree_size,
                "goal_tree_size": r.goal_tree_size}

    unsolved = [desc(i, x) for i, x in enumerate(results) if not x.solved]
    tail = {"last": desc(last, r), "unsolved": unsolved[:16], "unsolved_count": len(unsolved),
            "status_legend": "0 sample budget (max_iters x num_new_configs) spent, 2 arena full, 3 time budget"}
    return bulk, tail


def h2d_bytes(qs):
    b = 0
    for q in qs:
        e = q.env
        b += 4 * (4 * len(e.spheres) + 8 * (len(e.capsules) + len(e.z_aligned_capsules)) +
                  16 * (len(e.cuboids) + len(e.z_aligned_cuboids)))
        b += 4 * (len(q.start) + len(q.goal)) + 24
    return b


def ours(args, rank, world):
    import torch
    from prrtc_gb300 import BatchSettings, Context, autotune, build, workloads
    build.build()
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    robot = workloads.WORKLOADS[args.workload][0]
    n = args.queries
    # K steps of n queries each, distinct seeds, streamed through one launch
    qs = workloads.make(args.workload, n * args.steps, seed0=shard_seed0(rank, n, args.steps))
    first = qs[:n]
    plan = settings_for(args.workload)
    ctx = Context(dev)
    envs = [ctx.upload_env(q.env) for q in qs]
    tuned = autotune.load(robot, args.workload)
    common = dict(use_graph=1, margin=MARGIN, time_budget_ns=GPU_BUDGET_NS, **tuned)
    stream = ctx.batch(robot, [(e, q.start, q.goal) for e, q in zip(envs, qs)],
                       BatchSettings(plan, max_active=n, **common), path_capacity=2048)
    single = ctx.batch(robot, [(e, q.start, q.goal) for e, q in zip(envs[:n], first)], BatchSettings(plan, **common),
                       path_capacity=2048)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=f"cuda:{dev}")
    # warm-up: the first step's batch on its own, W times (also the one-batch figures)
    single_ms, single_solved = [], []
    for _ in range(args.warmup):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        single.run()
        res1 = single.results()
        single_ms.append(single.stats()["kernel_ns"] / 1e6)
        single_solved.append(sum(r.solved for r in res1))
    if world > 1:
        torch.distributed.barrier()
    flush.fill_(1.0)
    torch.cuda.synchronize()
    launches0 = ctx.launches
    with ClockSampler(dev) as clk:
        stream.run()
        torch.cuda.synchronize()
    launches = ctx.launches - launches0
    st = stream.stats()
    results = stream.results()
    solved = sum(r.solved for r in results)
    t_dev = st["kernel_ns"] * 1e-9
    bulk, tail = bulk_and_tail(results)
    t_dev, solved = reduce_over_ranks(t_dev, solved, world, f"cuda:{dev}")
    value = solved / t_dev
    lat = [r.kernel_ns / 1e6 for r in results if r.solved]
    if args.kernel_only:
        # a profiling run: the planner launches above and nothing else
        if rank == 0:
            print(json.dumps({"kernel_only": True, "queries": len(qs), "solved": solved, "ms": t_dev * 1e3,
                              "flops": st["flops"], "bulk_ms": st["bulk_ns"] / 1e6}), flush=True)
        return

    # ---- e2e through the C ABI with host buffers (same streamed job): the
    # prrtc_query array points at host start, goal and obstacle arrays, as a C
    # or C++ caller's would; the timed call uploads them, runs the batch and
    # copies results and paths back into host buffers
    host_q = [(q.env, q.start, q.goal) for q in qs]
    bs_host = BatchSettings(plan, max_active=n, **common)
    ctx.solve_batch(robot, host_q[:64], BatchSettings(plan, **common))
    torch.cuda.synchronize()
    prep = ctx.prepare_batch(robot, host_q, path_capacity=2048)
    # the caller's path buffers (n x 2048 rows, freshly allocated) are written
    # once here so that the timed call does not pay the operating system's
    # first-touch zeroing of their pages (64 KB pages on the GPU machine: ~40 ms
    # for this job), as a caller that reuses its buffers would not
    prep.paths.fill(0.0)
    t0 = time.perf_counter()
    ctx.solve_prepared(prep, bs_host)
    e2e_t = time.perf_counter() - t0
    res_e2e = prep.results()
    e2e_solved = sum(r.solved for r in res_e2e)
    d2h = sum(len(r.path) * r.path.shape[1] * 4 for r in res_e2e) + 64 * len(res_e2e)
    h2d = h2d_bytes(qs)
    # whole job over ranks: the slowest rank's call, all ranks' queries and bytes
    (e2e_t,), (e2e_solved, d2h, h2d) = allreduce([e2e_t], [e2e_solved, d2h, h2d], world, f"cuda:{dev}")
    # the same job through the Python wrapper (marshalling and unpacking timed)
    t0 = time.perf_counter()
    res_py = ctx.solve_batch(robot, host_q, bs_host, path_capacity=2048)
    e2e_py_t = time.perf_counter() - t0
    e2e_py_solved = sum(r.solved for r in res_py)

    if rank != 0:
        return
    # ---- revalidation of every returned path by the oracle checker
    O = oracle_lib()
    g = plan.granularity
    bad = sum(1 for q, r in zip(qs, results)
              if r.solved and not O.check_edges(robot, q.env, r.path[:-1], r.path[1:], g).all())

    # ---- distributional comparison on the first DIST_QUERIES queries of the
    # timed run: batched (this run's results), plain (the drop-in) and the
    # oracle's rrtc on the host cores; the plain and CPU figures below are
    # this leg's
    dist = {args.workload: distribution_leg(ctx, O, args.workload, qs, envs, batched=results)}
    plain_row = dist[args.workload]["plain_gpu"]
    plain_qps = plain_row["queries_per_s"]
    cpu_row = dist[args.workload]["oracle_cpu"]

    # ---- roofline: FP32 work of the planner kernel vs the measured FP32 peak
    peak = ctx.measure_fp32_peak()
    achieved = st["flops"] / (st["kernel_ns"] * 1e-9) / 1e12
    nn_bytes = st["nn_nodes"] * 4 * plan_dof(robot)

    # ---- the other configurations, one launch each; the tabletop one also
    # gets the distributional comparison (its first DIST_QUERIES queries)
    others, baxter = {}, None
    if args.others:
        for name, cnt in OTHER_WORKLOADS:
            if name == args.workload:
                continue
            info, run = workload_run(ctx, O, name, cnt)
            others[f"{name}_{cnt}"] = info
            if name == "baxter_mixed":
                baxter = run
            if name == "panda_tabletop":
                oq, ores, oenvs = run
                dist[name] = distribution_leg(ctx, O, name, oq, oenvs, batched=ores)
            log(name, json.dumps(info))

    # ---- the stand-alone checker (validator) on the C0 and C1 scenes
    validator = validator_leg(ctx, peak) if args.validator else None

    # ---- differentiable clearance: smoothing of this run's paths (and Baxter's)
    clearance = None
    if args.clearance and robot == "panda":
        clearance = clearance_leg(ctx, O, qs, results, envs, baxter)

    clocks = clk.summary()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    theo = sm_count * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12 if clocks.get("sm_mhz") else None
    single_med = statistics.median(single_ms)
    line = {
        "metric": metric_name(args), "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_of(args),
        "p50_solve_ms": statistics.median(lat) if lat else None,
        "p99_solve_ms": float(np.percentile(lat, 99)) if lat else None,
        "max_solve_ms": max(lat) if lat else None,
        "success_rate": solved / len(qs), "revalidated": f"{solved - bad}/{solved}",
        "edge_validations_per_s": st["configs_checked"] / g / (st["kernel_ns"] * 1e-9),
        "configs_per_s": st["configs_checked"] / (st["kernel_ns"] * 1e-9),
        "extra_attempts": st["extra_attempts"],
        "one_batch": {"queries": n, "ms_median": single_med, "ms_all": single_ms,
                      "queries_per_s": statistics.median(single_solved) / (single_med * 1e-3),
                      "note": "the first step's queries alone in one launch: its time is its slowest query's"},
        "bulk": bulk,
        "tail": tail,
        "plain": {"queries_per_s": plain_qps, "p50_solve_ms": plain_row["p50_solve_ms"],
                  "success_rate": plain_row["success_rate"],
                  "sample": f"the first {DIST_QUERIES} queries of the timed run, one at a time",
                  "batched_over_plain": value / plain_qps if plain_qps else None,
                  "batched_bulk_over_plain": bulk["queries_per_s"] / plain_qps if bulk and plain_qps else None},
        "distribution": dist,
        "validator": validator,
        "e2e": {"value": e2e_solved / e2e_t, "unit": "queries/s", "h2d_bytes_per_step": int(h2d) // args.steps,
                "d2h_bytes_per_step": int(d2h) // args.steps, "call_ms": e2e_t * 1e3,
                "create_ms": res_e2e[0].copy_ns / 1e6 if res_e2e else None,
                "launch_ms": max((r.finish_ns for r in res_e2e), default=0) / 1e6,
                "split": "call_ms = create_ms (packing and upload) + launch_ms (this call's own launch, "
                         "from its start to the last query's end; its tail varies from run to run like "
                         "the device-timed launch's) + result copies, unpacking and release",
                "buffers": "prrtc_query / prrtc_result arrays and the path buffers prepared, and the path "
                           "buffers' pages touched, before the timed call"},
        "e2e_python": {"value": e2e_py_solved / e2e_py_t, "unit": "queries/s",
                       "note": "Context.solve_batch: the Python wrapper's marshalling and unpacking included"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "peak_theoretical": theo, "frac_theoretical": achieved / theo if theo else None,
                     "peak_theoretical_source": "SMs x 128 FP32 lanes x 2 FLOP x the median SM clock sampled "
                                                "during the timed launch",
                     "traffic": (lambda b: b * len(qs) if b else None)(profiled_dram_bytes_per_query(args.workload)),
                     "traffic_source": "ncu capture of 256 queries (profiles/), scaled by queries processed",
                     "peak_source": "measured FP32 FMA chain kernel on this GPU (prrtc_measure_fp32_peak)",
                     "nn_scan_bytes_per_s": nn_bytes / (st["kernel_ns"] * 1e-9),
                     "nn_scan_tflops": 3 * plan_dof(robot) * st["nn_nodes"] / (st["kernel_ns"] * 1e-9) / 1e12,
                     "nn_scan_note": "nearest-node passes: 4 D bytes and 3 D FLOPs per node visited and sample; "
                                     "32 nodes of each tree are staged per step in shared memory and serve all "
                                     "32 samples of a round, from L2 (the trees stay L2-resident)",
                     "bulk": ({"achieved": st["bulk_flops"] / (st["bulk_ns"] * 1e-9) / 1e12,
                               "frac": st["bulk_flops"] / (st["bulk_ns"] * 1e-9) / 1e12 / peak,
                               "ms": st["bulk_ns"] / 1e6,
                               "note": "the launch up to the moment 99 % of its queries had finished"}
                              if st["bulk_ns"] else None)},
        "cpu_baseline": {"value": cpu_row["queries_per_s"], "unit": "queries/s", "cores": cpu_row["threads"],
                         "kind": "port",
                         "sample": f"the first {DIST_QUERIES} of the {len(qs)} queries, oracle RRT-Connect "
                                   f"restatement, {DIST_CPU_BUDGET_S:.0f} s per query"},
        "gpu_launches": launches,
        "clocks": clocks,
        "other_workloads": others or None,
        "clearance": clearance,
    }
    print(json.dumps(line), flush=True)


DIST_QUERIES = 256          # seeds per configuration in the distributional comparison
DIST_CPU_BUDGET_S = 10.0    # per query, the oracle's rrtc on the host cores
DIST_PLAIN_BUDGET_NS = int(5e9)   # per query, the plain form


def quantiles(costs):
    if not len(costs):
        return None
    c = np.asarray(costs, np.float64)
    return {"p10": float(np.percentile(c, 10)), "p50": float(np.percentile(c, 50)), "p90": float(np.percentile(c, 90))}


def distribution_leg(ctx, O, name, qs, envs, batched=None):
    """Success rate and path-cost quantiles over the same DIST_QUERIES seeded
    queries for three planners: the GPU batched form, the GPU plain form (the
    drop-in, one query at a time, with pRRTC's own lane count) and the
    oracle's restatement of pRRTC's rrtc on the host cores (the reference
    algorithm; OpenMP over queries, DIST_CPU_BUDGET_S per query).  Cost is
    pRRTC's: the summed length of the traced edges (pRRTC.cu:561,571).
    `batched`: results of these queries from a run already made, else one
    batch launch here."""
    from prrtc_gb300 import BatchSettings, autotune, workloads
    robot = workloads.WORKLOADS[name][0]
    plan = settings_for(name)
    qs, envs = qs[:DIST_QUERIES], envs[:DIST_QUERIES]
    n = len(qs)
    if batched is None:
        batched = ctx.solve_batch(robot, [(e, q.start, q.goal) for e, q in zip(envs, qs)],
                                  BatchSettings(plan, use_graph=0, margin=MARGIN, time_budget_ns=GPU_BUDGET_NS,
                                                **autotune.load(robot, name)), path_capacity=2048)
    batched = batched[:n]
    ctx.set_planning_margin(MARGIN)
    ctx.set_time_budget(DIST_PLAIN_BUDGET_NS)
    plain, plain_t = [], 0.0
    for q, e in zip(qs, envs):
        r = ctx.solve(robot, q.start, q.goal, e, plan)
        plain.append(r)
        plain_t += r.wall_ns * 1e-9
    g = plan.granularity
    plain_bad = sum(1 for q, r in zip(qs, plain)
                    if r.solved and not O.check_edges(robot, q.env, r.path[:-1], r.path[1:], g).all())
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ores, _ = O.solve_many(robot, np.stack([q.start for q in qs]), np.stack([q.goal for q in qs]),
                           [q.env for q in qs], plan, threads=threads, path_cap=16, budget_s=DIST_CPU_BUDGET_S)
    cpu_t = time.perf_counter() - t0

    def row(res, extra=None):
        solved = [r for r in res if r.solved]
        d = {"success_rate": len(solved) / n, "cost": quantiles([r.cost for r in solved])}
        d.update(extra or {})
        return d

    lat = [r.wall_ns / 1e6 for r in plain if r.solved]
    out = {"queries": n, "settings": WORKLOAD_SETTINGS[name],
           "batched_gpu": row(batched),
           "plain_gpu": row(plain, {"queries_per_s": sum(r.solved for r in plain) / plain_t,
                                    "p50_solve_ms": statistics.median(lat) if lat else None,
                                    "revalidated": f"{sum(r.solved for r in plain) - plain_bad}/"
                                                   f"{sum(r.solved for r in plain)}",
                                    "budget_s": DIST_PLAIN_BUDGET_NS * 1e-9}),
           "oracle_cpu": row(ores, {"queries_per_s": sum(r.solved for r in ores) / cpu_t, "threads": threads,
                                    "budget_s": DIST_CPU_BUDGET_S, "wall_s": cpu_t}),
           "note": "batched: margin 1e-5 m, tuned lanes; plain: pRRTC's settings and lane count, margin 1e-5 m; "
                   "oracle: pRRTC's rrtc restated (lanes round-robin), margin 0"}
    log("distribution", name, json.dumps(out))
    return out


def smooth_and_judge(ctx, O, robot, envs, hosts, P):
    """prrtc_smooth_paths on device-resident paths P [n, 64, dof] (timed), then
    every accepted path re-checked by the oracle at 128 points per edge."""
    import torch
    from prrtc_gb300 import SmoothSettings, paths
    s = SmoothSettings()
    ctx.smooth_paths(robot, envs[:8], torch.from_numpy(P[:8]).cuda(), s)        # warm-up (tables, attribute)
    q = torch.from_numpy(P).cuda()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q, acc, cb, ca = ctx.smooth_paths(robot, envs, q, s)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out, acc, cb, ca = q.cpu().numpy(), acc.cpu().numpy().astype(bool), cb.cpu().numpy(), ca.cpu().numpy()
    bad = sum(1 for i in np.flatnonzero(acc)
              if not O.check_edges(robot, hosts[i], out[i, :-1], out[i, 1:], s.granularity).all())
    return {"paths": len(P), "ms": dt * 1e3, "paths_per_s": len(P) / dt, "accepted": int(acc.sum()),
            "accepted_revalidated": f"{int(acc.sum()) - bad}/{int(acc.sum())}",
            "cost_before": float(cb[acc].sum()), "cost_after": float(ca[acc].sum()),
            "length_before": float(paths.length(P[acc]).sum()), "length_after": float(paths.length(out[acc]).sum())}


def resampled(qs, results, envs, n):
    from prrtc_gb300 import paths
    E, H, P = [], [], []
    for q, r, e in zip(qs, results, envs):
        if r.solved:
            p = paths.resample(paths.start_first(r.path), 64)
            if p is not None:
                E.append(e)
                H.append(q.env)
                P.append(p)
        if len(P) == n:
            break
    return E, H, np.stack(P)


def clearance_leg(ctx, O, qs, results, envs, baxter):
    """Differentiable clearance: 4096 Panda paths of this run and 1024 Baxter
    paths (tabletop and shelf scenes) resampled to 64 waypoints, margin 0.02 m,
    50 smoothing steps, the checker as judge."""
    out = {"config": "paths resampled to 64 waypoints (planner vertices kept), margin 0.02 m, 50 steps, "
                     "judged at 128 points per edge by the robot's checker, then re-checked by the oracle"}
    E, H, P = resampled(qs, results, envs, 4096)
    out["panda"] = smooth_and_judge(ctx, O, "panda", E, H, P)
    if baxter is not None:
        E, H, P = resampled(*baxter, 1024)
        out["baxter"] = smooth_and_judge(ctx, O, "baxter", E, H, P)
    return out


# the other configurations: one launch of n queries each (after one warm-up launch)
OTHER_WORKLOADS = [("panda_tabletop", 1024), ("fetch_mixed", 256), ("baxter_mixed", 1024)]


OTHER_BUDGET_NS = int(10e9)   # per launch of the other configurations


def workload_run(ctx, O, name, n):
    """One batched launch of workload `name` (after a warm-up launch of its
    first 32 queries): solved queries/s over the launch, the bulk rate and
    tail (bulk_and_tail), solve-time percentiles, edge validations/s, every
    path revalidated by the oracle.  A launch whose unsolved queries run into
    the time budget lasts the budget; the tail says which queries and why."""
    from prrtc_gb300 import BatchSettings, autotune, workloads
    robot = workloads.WORKLOADS[name][0]
    qs = workloads.make(name, n)
    envs = [ctx.upload_env(q.env) for q in qs]
    plan = settings_for(name)
    bs = BatchSettings(plan, use_graph=1, margin=MARGIN, time_budget_ns=OTHER_BUDGET_NS, **autotune.load(robot, name))
    ctx.solve_batch(robot, [(e, q.start, q.goal) for e, q in zip(envs[:32], qs[:32])], bs)
    b = ctx.batch(robot, [(e, q.start, q.goal) for e, q in zip(envs, qs)], bs, path_capacity=2048)
    b.run()
    st, res = b.stats(), b.results()
    b.free()
    t = st["kernel_ns"] * 1e-9
    solved = sum(r.solved for r in res)
    g = plan.granularity
    bad = sum(1 for q, r in zip(qs, res) if r.solved and not O.check_edges(robot, q.env, r.path[:-1], r.path[1:], g).all())
    lat = [r.kernel_ns / 1e6 for r in res if r.solved]
    bulk, tail = bulk_and_tail(res)
    info = {"queries": n, "settings": WORKLOAD_SETTINGS[name], "queries_per_s": solved / t, "ms": t * 1e3,
            "success_rate": solved / n, "revalidated": f"{solved - bad}/{solved}",
            "budget_s": OTHER_BUDGET_NS * 1e-9, "unsolved_in_budget": n - solved, "bulk": bulk, "tail": tail,
            "p50_solve_ms": statistics.median(lat) if lat else None,
            "p90_solve_ms": float(np.percentile(lat, 90)) if lat else None,
            "p99_solve_ms": float(np.percentile(lat, 99)) if lat else None,
            "edge_validations_per_s": st["configs_checked"] / g / t,
            "configs_per_s": st["configs_checked"] / t,
            "fp32_tflops": st["flops"] / t / 1e12}
    return info, (qs, res, envs)


VALIDATOR_SCENES = [("C0 panda tabletop (seed 0)", "tabletop", 0, 32), ("C1 panda shelf (seed 1)", "shelf", 1, 128)]
VALIDATOR_N = 1 << 20
VALIDATOR_EDGES = 1 << 14
VALIDATOR_REPS = 5


def validator_leg(ctx, peak):
    """The stand-alone checker (prrtc_validate_configs / prrtc_validate_edges)
    on the C0 and C1 scenes: 2^20 configurations, uniformly random and
    collision-free, and 2^14 edges between collision-free configurations at
    the scene's granularity.  Inputs are resident on the device; each launch
    is timed with CUDA events on the library's stream (prrtc_last_kernel_ns),
    a 256 MB write flushes L2 before each, and the median of 5 is reported.
    FLOPs are the checker's counted algorithmic work (the reference
    hierarchy's executed tests x weights + canonical FK)."""
    import torch
    from prrtc_gb300 import scenes
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    out = {"peak_tflops": peak, "configs": VALIDATOR_N, "edges": VALIDATOR_EDGES, "reps": VALIDATOR_REPS}

    def timed(fn):
        ms, fl = [], []
        for _ in range(VALIDATOR_REPS):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ctx.work_counters(reset=True)
            fn()
            ms.append(ctx.last_kernel_ns() / 1e6)
            fl.append(ctx.work_counters(reset=True)[0])
        k = int(np.argsort(ms)[len(ms) // 2])
        return ms[k], fl[k]

    for label, kind, seed, g in VALIDATOR_SCENES:
        env = scenes.make_query("panda", kind, seed).env
        e = ctx.upload_env(env)
        rnd = scenes._uniform_configs("panda", scenes.Rng(4242 + seed), VALIDATOR_N)
        q = torch.from_numpy(rnd).cuda()
        free = ctx.validate_configs("panda", e, q).cpu().numpy().astype(bool)
        fq = rnd[free]
        fq = np.resize(fq, (VALIDATOR_N, 7)) if len(fq) else rnd
        qf = torch.from_numpy(np.ascontiguousarray(fq)).cuda()
        rows = {}
        for name, qq in (("random", q), ("collision_free", qf)):
            ms, fl = timed(lambda: ctx.validate_configs("panda", e, qq))
            rows[name] = {"ms": ms, "configs_per_s": VALIDATOR_N / (ms * 1e-3),
                          "tflops": fl / (ms * 1e-3) / 1e12, "frac": fl / (ms * 1e-3) / 1e12 / peak}
        rows["random"]["free_fraction"] = float(free.mean())
        a = torch.from_numpy(np.ascontiguousarray(fq[:VALIDATOR_EDGES])).cuda()
        b = torch.from_numpy(np.ascontiguousarray(np.roll(fq, 1, axis=0)[:VALIDATOR_EDGES])).cuda()
        ms, fl = timed(lambda: ctx.validate_edges("panda", e, a, b, g))
        rows["edges"] = {"granularity": g, "ms": ms, "edge_validations_per_s": VALIDATOR_EDGES / (ms * 1e-3),
                         "configs_per_s": VALIDATOR_EDGES * g / (ms * 1e-3), "tflops": fl / (ms * 1e-3) / 1e12,
                         "frac": fl / (ms * 1e-3) / 1e12 / peak}
        out[label] = rows
        log("validator", label, json.dumps(rows))
    return out


def profiled_dram_bytes_per_query(workload: str):
    """DRAM bytes per query of k_rrtc_batch from the committed ncu summary of a
    smaller case of this workload (traffic scales with the queries processed)."""
    import re
    f = ROOT / "profiles" / f"k_rrtc_batch_{workload}.md"
    if not f.exists():
        return None
    m = re.search(r"dram_bytes_per_query \| (\d+)", f.read_text())
    return int(m.group(1)) if m else None


def plan_dof(robot):
    return {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="panda_shelf", choices=sorted(WORKLOAD_SETTINGS))
    ap.add_argument("--queries", type=int, default=1024)
    ap.add_argument("--no-clearance", dest="clearance", action="store_false",
                    help="skip the path-smoothing measurement")
    ap.add_argument("--no-others", dest="others", action="store_false",
                    help="skip the other configurations (Panda tabletop, Fetch, Baxter: one launch each, "
                         "parity cases beside the benchmark)")
    ap.add_argument("--no-validator", dest="validator", action="store_false",
                    help="skip the stand-alone checker measurement")
    ap.add_argument("--kernel-only", action="store_true",
                    help="run the warm-up and timed planner launches only and print a short line (for profilers)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # started without a launcher: one rank per GPU on this node
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()),
               *sys.argv[1:]]
        sys.exit(subprocess.call(cmd))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if world > 1:
        import torch
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group(backend)
    if args.impl == "reference":
        reference_arm(args, rank, world)
    else:
        ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
