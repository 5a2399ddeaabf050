"""Named benchmark workloads (lists of seeded queries), built in parallel and
cached on disk (``$PRRTC_CACHE``, default /tmp/prrtc_workloads)."""
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


def _one(args):
    robot, kind, seed, nobs, z = args
    if kind == "mixed":
        nobs = 5 + scenes.Rng(seed ^ 0x77).integers(0, 55) if nobs is None else nobs
        return scenes.make_query(robot, kind, seed, nobs)
    return scenes.make_query(robot, kind, seed, z_offset=z)


def make(name: str, n: int, seed0: int = 0, procs: int | None = None) -> list:
    robot, kinds, z = WORKLOADS[name]
    cache = Path(os.environ.get("PRRTC_CACHE", "/tmp/prrtc_workloads"))
    f = cache / f"{name}_{n}_{seed0}.pkl"
    if f.exists():
        with open(f, "rb") as fh:
            return pickle.load(fh)
    args = [(robot, kinds[i % len(kinds)][0], seed0 + i, kinds[i % len(kinds)][1], z) for i in range(n)]
    procs = procs or min(16, os.cpu_count() or 1)
    if procs > 1 and n > 8:
        with ProcessPoolExecutor(procs, mp_context=get_context("spawn")) as ex:
            qs = list(ex.map(_one, args, chunksize=max(1, n // (4 * procs))))
    else:
        qs = [_one(a) for a in args]
    cache.mkdir(parents=True, exist_ok=True)
    tmp = f.with_suffix(".tmp")
    with open(tmp, "wb") as fh:
        pickle.dump(qs, fh)
    tmp.replace(f)
    return qs
