"""Per-robot autotuner of the batched planner's launch and work shape.

Sweeps, on a calibration batch of seeded queries, the knobs of
``prrtc_batch_settings`` that change speed but not answers' validity:

* ``warps_per_block``  block size (warps are independent workers);
* ``lanes``            virtual sampling lanes per query (samples per
                       iteration round of a query);
* ``edge_order``       edge tile shape: contiguous 32-point rounds or rounds
                       interleaved across the whole edge;
* ``sampler``          the reference's Halton lanes or per-query scrambled
                       Halton;
* ``max_workers_per_attempt``  warps per attempt before idle warps open
                       independent attempts (the tail's portfolio);
* ``max_attempts``     attempts per query, 1 (pRRTC's behaviour: a query whose
                       attempt fails stays unsolved) or 4 (an attempt that
                       exhausts its samples or arena restarts the query);

and keeps the setting with the highest solved queries per second among those
that solve the most queries.  Results are cached in ``tuning.json`` next to
this file, keyed by robot and workload; each entry's ``source`` says whether
its ``best`` is the sweep's winner ("sweep") or was set by hand after
longer measurements than the sweep makes ("hand-set", with a ``note``):

    python -m prrtc_gb300.autotune panda_shelf [queries] [budget_s]   # on a GPU; rewrites the entry
"""
from __future__ import annotations

import itertools
import json
import sys
from pathlib import Path

TUNING = Path(__file__).resolve().parent / "tuning.json"
DEFAULT = {"lanes": 1, "warps_per_block": 2, "edge_order": 0, "sampler": 0, "max_workers_per_attempt": 0,
           "max_attempts": 4}
SPACE = {"lanes": (1, 2), "warps_per_block": (2, 4), "edge_order": (0, 1), "sampler": (0, 1),
         "max_workers_per_attempt": (64, 0), "max_attempts": (1, 4)}
KNOBS = tuple(SPACE)


def load(robot: str, workload: str | None = None) -> dict:
    """Tuned knobs for (robot, workload), else the robot's best entry, else defaults."""
    if TUNING.exists():
        table = json.loads(TUNING.read_text())
        if workload and f"{robot}/{workload}" in table:
            return dict(table[f"{robot}/{workload}"]["best"])
        for k, v in table.items():
            if k.startswith(robot + "/"):
                return dict(v["best"])
    return dict(DEFAULT)


def tune(ctx, robot, queries, plan, margin=1e-5, reps=3, space=None, budget_ns=int(60e9)) -> dict:
    """Run every setting `reps` times and keep the one with the best median
    batch time among those that solve the most queries.  With a time budget
    shorter than the batch needs, the most queries solved within it decides."""
    import statistics
    from .api import BatchSettings
    space = space or SPACE
    rows = []
    for values in itertools.product(*(space[k] for k in KNOBS)):
        knobs = dict(zip(KNOBS, values))
        bs = BatchSettings(plan, use_graph=1, margin=margin, time_budget_ns=budget_ns, **knobs)
        b = ctx.batch(robot, queries, bs)
        b.run()
        times, solved = [], []
        for _ in range(reps):
            b.run()
            res = b.results()
            times.append(b.stats()["kernel_ns"] * 1e-6)
            solved.append(sum(r.solved for r in res))
        b.free()
        med = statistics.median(times)
        rows.append({**knobs, "ms_median": med, "ms_all": times, "solved": min(solved),
                     "queries_per_s": min(solved) / (med * 1e-3)})
    top = max(r["solved"] for r in rows)
    best = max((r for r in rows if r["solved"] == top), key=lambda r: r["queries_per_s"])
    return {"best": {k: best[k] for k in KNOBS}, "source": "sweep", "sweep": rows}


def main(argv):
    from . import workloads
    from .api import Context, Settings
    name = argv[1] if len(argv) > 1 else "panda_shelf"
    n = int(argv[2]) if len(argv) > 2 else 1024
    budget_s = float(argv[3]) if len(argv) > 3 else 60.0
    robot = workloads.WORKLOADS[name][0]
    qs = workloads.make(name, n, seed0=100_000)    # calibration queries, disjoint from the benchmark's
    ctx = Context(0)
    envs = [ctx.upload_env(q.env) for q in qs]
    out = tune(ctx, robot, [(e, q.start, q.goal) for e, q in zip(envs, qs)], Settings(**workloads.SETTINGS[name]),
               budget_ns=int(budget_s * 1e9))
    table = json.loads(TUNING.read_text()) if TUNING.exists() else {}
    table[f"{robot}/{name}"] = out
    TUNING.write_text(json.dumps(table, indent=1) + "\n")
    print(json.dumps(out["best"]), file=sys.stderr)
    for r in out["sweep"]:
        print(r, file=sys.stderr)


if __name__ == "__main__":
    main(sys.argv)
