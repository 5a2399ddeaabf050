"""Per-robot autotuner of the batched planner's launch and work shape.

Sweeps, on a calibration batch of seeded queries, the knobs of
``prrtc_batch_settings`` that change speed but not answers' validity:

* ``warps_per_block``  block size (warps are independent workers);
* ``lanes``            virtual sampling lanes per query (samples per
                       iteration round of a query);
* ``edge_order``       edge tile shape: contiguous 32-point rounds or rounds
                       interleaved across the whole edge;

and keeps the setting with the highest solved queries per second.  Results
are cached in ``tuning.json`` next to this file, keyed by robot and workload:

    python -m prrtc_gb300.autotune panda_shelf [queries]   # on a GPU; rewrites the entry
"""
from __future__ import annotations

import itertools
import json
import sys
from pathlib import Path

TUNING = Path(__file__).resolve().parent / "tuning.json"
DEFAULT = {"lanes": 2, "warps_per_block": 4, "edge_order": 1}
SPACE = {"lanes": (1, 2, 4), "warps_per_block": (2, 4), "edge_order": (0, 1)}


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


def tune(ctx, robot, queries, plan, margin=1e-5, reps=2, space=None) -> dict:
    from .api import BatchSettings
    space = space or SPACE
    rows = []
    for lanes, wpb, order in itertools.product(space["lanes"], space["warps_per_block"], space["edge_order"]):
        bs = BatchSettings(plan, lanes=lanes, warps_per_block=wpb, edge_order=order, use_graph=1, margin=margin)
        b = ctx.batch(robot, queries, bs)
        b.run()
        ns, solved = 0, 0
        for _ in range(reps):
            b.run()
            res = b.results()
            ns += b.stats()["kernel_ns"]
            solved += sum(r.solved for r in res)
        b.free()
        rows.append({"lanes": lanes, "warps_per_block": wpb, "edge_order": order,
                     "queries_per_s": solved / (ns * 1e-9), "ms_per_batch": ns / reps / 1e6})
    best = max(rows, key=lambda r: r["queries_per_s"])
    return {"best": {k: best[k] for k in ("lanes", "warps_per_block", "edge_order")}, "sweep": rows}


def main(argv):
    from . import workloads
    from .api import Context, Settings
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from bench import WORKLOAD_SETTINGS   # the benchmark's settings per workload
    name = argv[1] if len(argv) > 1 else "panda_shelf"
    n = int(argv[2]) if len(argv) > 2 else 1024
    robot = workloads.WORKLOADS[name][0]
    qs = workloads.make(name, n, seed0=10_000)     # calibration queries, disjoint from the benchmark's
    ctx = Context(0)
    envs = [ctx.upload_env(q.env) for q in qs]
    out = tune(ctx, robot, [(e, q.start, q.goal) for e, q in zip(envs, qs)], Settings(**WORKLOAD_SETTINGS[name]))
    table = json.loads(TUNING.read_text()) if TUNING.exists() else {}
    table[f"{robot}/{name}"] = out
    TUNING.write_text(json.dumps(table, indent=1) + "\n")
    print(json.dumps(out["best"]), file=sys.stderr)
    for r in out["sweep"]:
        print(r, file=sys.stderr)


if __name__ == "__main__":
    main(sys.argv)
