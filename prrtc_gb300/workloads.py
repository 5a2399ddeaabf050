"""Named benchmark workloads (lists of seeded queries), built in parallel.

Building a workload is deterministic, so a cache is only a speed-up: when
``$PRRTC_CACHE`` names a directory, built workloads are pickled there and
read back on the next call; otherwise nothing is written to disk."""
from __future__ import annotations

import os
import pickle
from concurrent.futures import ProcessPoolExecutor
from multiprocessing import get_context
from pathlib import Path

from . import scenes

# name -> (robot, [(kind, n_obstacles or None)] cycled over queries, z_offset)
WORKLOADS = {
    "panda_tabletop": ("panda", [("tabletop", None)], 0.0),
    "panda_shelf": ("panda", [("shelf", None)], 0.0),
    "fetch_mixed": ("fetch", [("mixed", None)], 0.0),
    "baxter_mixed": ("baxter", [("tabletop", None), ("shelf", None)], 0.3),
}

# planner settings of each workload (pRRTC_settings fields; others default)
SETTINGS = {
    # Panda shelf: granularity 128, balance 2, tree_ratio 1, dynamic domain (radius 4, alpha 1e-4, min 1)
    "panda_shelf": dict(granularity=128, balance=2, tree_ratio=1.0, dynamic_domain=True, dd_radius=4.0,
                        dd_alpha=1e-4, dd_min_radius=1.0),
    # Panda tabletop: range 1.0, granularity 32, 256 lanes, 100k samples, balance 0, dynamic domain off
    "panda_tabletop": dict(max_samples=100000, num_new_configs=256, granularity=32, range=1.0, balance=0,
                           dynamic_domain=False),
    "fetch_mixed": dict(granularity=64),
    "baxter_mixed": dict(granularity=128, balance=1, tree_ratio=0.5),
}


def _one(args):
    robot, kind, seed, nobs, z = args
    if kind == "mixed":
        nobs = 5 + scenes.Rng(seed ^ 0x77).integers(0, 55) if nobs is None else nobs
        return scenes.make_query(robot, kind, seed, nobs)
    return scenes.make_query(robot, kind, seed, z_offset=z)


def make(name: str, n: int, seed0: int = 0, procs: int | None = None) -> list:
    robot, kinds, z = WORKLOADS[name]
    cache = Path(os.environ["PRRTC_CACHE"]) if os.environ.get("PRRTC_CACHE") else None
    f = cache / f"{name}_{n}_{seed0}.pkl" if cache else None
    if f is not None and f.exists():
        with open(f, "rb") as fh:
            return pickle.load(fh)
    args = [(robot, kinds[i % len(kinds)][0], seed0 + i, kinds[i % len(kinds)][1], z) for i in range(n)]
    procs = procs or min(16, os.cpu_count() or 1)
    if procs > 1 and n > 8:
        with ProcessPoolExecutor(procs, mp_context=get_context("spawn")) as ex:
            qs = list(ex.map(_one, args, chunksize=max(1, n // (4 * procs))))
    else:
        qs = [_one(a) for a in args]
    if f is None:
        return qs
    cache.mkdir(parents=True, exist_ok=True)
    tmp = f.with_suffix(".tmp")
    with open(tmp, "wb") as fh:
        pickle.dump(qs, fh)
    tmp.replace(f)
    return qs
