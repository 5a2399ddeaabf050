"""Generate the golden fixtures in this directory from the reference itself.

Run where a pRRTC checkout is available (its path as the argument, else
$PRRTC_REFERENCE):

    make -C oracle ref REF=/path/to/pRRTC   # pRRTC's own checker, from its sources
    python tests/golden/make_golden.py [/path/to/pRRTC]

For each robot and scene it writes checker_<robot>_<scene>.npz with
  env_*      the obstacle arrays (flat C-ABI layouts)
  q          seeded configurations (uniform within the joint limits, plus
             points on segments between them so that many lie near contact)
  free_ref   pRRTC's own fkcc<Robot> verdicts (host build of utils.cuh)
  margin     the oracle's float64 near-contact measure for each config
  fk_q, fk_centres   a subset of q and every model sphere's centre from the
             float64 evaluation of the reference's generated FK code
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from prrtc_gb300 import scenes  # noqa: E402
from prrtc_gb300.robots import extract, refparse  # noqa: E402
from pyoracle import OracleLib, RefLib  # noqa: E402

CASES = [("sphere", "tabletop", 11), ("panda", "tabletop", 0), ("panda", "shelf", 1), ("fetch", "mixed", 2),
         ("baxter", "tabletop", 3), ("baxter", "shelf", 4),
         # scenes holding z-aligned capsules and z-aligned cuboids as well
         ("sphere", "zmixed", 12), ("panda", "ztabletop", 5), ("panda", "zshelf", 6), ("fetch", "zmixed", 7),
         ("baxter", "zmixed", 8)]
N_UNIFORM, N_SEGMENT, N_FK = 3072, 1024, 64


def configs(robot: str, seed: int) -> np.ndarray:
    rng = np.random.default_rng(1000 + seed)
    sc, off = (np.array(v) for v in scenes.LIMITS[robot])
    u = rng.random((N_UNIFORM, len(sc))) * sc + off
    a = rng.random((N_SEGMENT, len(sc))) * sc + off
    b = rng.random((N_SEGMENT, len(sc))) * sc + off
    t = rng.random((N_SEGMENT, 1))
    return np.concatenate([u, a + t * (b - a)]).astype(np.float32)


def scene(robot, kind, seed):
    """The fixture's obstacles.  A 'z' prefix adds z-aligned obstacles
    (vertical capsules, yawed boxes): 20 for the sphere robot, 12 in mixed
    clutter, 8 on a table, 6 in shelf cells."""
    nz = 0
    if kind.startswith("z"):
        kind = kind[1:]
        nz = {"mixed": 12, "tabletop": 8, "shelf": 6}[kind]
    if robot == "sphere":
        return scenes.mixed_scene(seed, 40, lo=(-4, -4, -4), hi=(4, 4, 4), n_zaligned=20 if nz else 0)
    if kind == "mixed":
        return scenes.mixed_scene(seed, 40, n_zaligned=nz)
    z = 0.3 if robot == "baxter" else 0.0
    if kind == "tabletop":
        return scenes.tabletop_scene(seed, z_offset=z, n_zaligned=nz)
    if robot == "baxter":
        return scenes.shelf_scene(seed, z_offset=z, n_zaligned=nz)
    return scenes.make_query(robot, kind, seed, n_zaligned=nz).env


def main(ref_root: str, force: bool = False):
    """Write every fixture that is missing (all of them with force)."""
    O, R = OracleLib(), RefLib()
    for robot, kind, seed in CASES:
        out = ROOT / "tests" / "golden" / f"checker_{robot}_{kind}.npz"
        if out.exists() and not force:
            continue
        env = scene(robot, kind, seed)
        q = configs(robot, seed)
        free_ref = R.check(robot, env, q)
        free_or, margin = O.check(robot, env, q, margin=True)
        bad = np.flatnonzero(free_ref != free_or)
        assert np.all(margin[bad] < 1e-5), "oracle disagrees with the reference away from contact"
        fk_q = q[:N_FK]
        if robot == "sphere":
            fk_c = np.stack([fk_q.astype(np.float64)], 0)
        else:
            prog = refparse.load_program(ref_root, robot)
            m = scenes.load_model(robot)
            keys, _ = extract._sphere_keys(prog)
            fk_c = extract._centres(prog, keys, fk_q.astype(np.float64))   # (S, N, 3) in the model's sphere order
            assert fk_c.shape[0] == len(m["spheres"])
        np.savez_compressed(out, env_spheres=env.spheres, env_capsules=env.capsules,
                            env_z_capsules=env.z_aligned_capsules, env_cuboids=env.cuboids,
                            env_z_cuboids=env.z_aligned_cuboids, q=q, free_ref=free_ref, margin=margin,
                            fk_q=fk_q, fk_centres=np.transpose(fk_c, (1, 0, 2)))
        print(f"{out.name}: {len(q)} configs, free {free_ref.mean():.3f}, oracle mismatches {len(bad)}, "
              f"near-contact (<1e-5 m) {(margin < 1e-5).sum()}")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--force"]
    if not args and not os.environ.get("PRRTC_REFERENCE"):
        sys.exit("usage: make_golden.py [--force] /path/to/pRRTC   (or set PRRTC_REFERENCE)")
    main(args[0] if args else os.environ["PRRTC_REFERENCE"], force="--force" in sys.argv)
