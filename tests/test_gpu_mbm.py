"""MotionBenchMaker-format problems through the GPU planner (scene I/O row).

No MBM data is stored or read: problems are written here in the MBM JSON
schema (spheres; cylinders with centre, Euler XYZ, radius and length; boxes
with centre, Euler XYZ and half-extents; start, goals, valid) from seeded
synthetic obstacles, saved as a problems file, read back by
prrtc_gb300.mbm.load_problems (the restatement of evaluate_mbm.cpp:13-86),
planned by the batched GPU planner and every path revalidated by the oracle.
Half the problems are in the `box` family, whose cylinders the reference's
loader turns into cuboids with half-extents (r, r, r/2) (evaluate_mbm.cpp:
27-39); the others keep them as capsules."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def synthetic_problem(seed: int, family: str) -> dict:
    from prrtc_gb300 import mbm, scenes
    rng = scenes.Rng(seed)
    lo, hi = np.array([0.4, -0.5, 0.3]), np.array([1.2, 0.5, 1.2])
    p = {"sphere": [], "cylinder": [], "box": [], "valid": True}
    for _ in range(6):
        p["sphere"].append({"position": [float(v) for v in rng.uniform(lo, hi, (3,))],
                            "radius": float(rng.uniform(0.03, 0.08))})
    for _ in range(6):
        p["cylinder"].append({"position": [float(v) for v in rng.uniform(lo, hi, (3,))],
                              "orientation_euler_xyz": [float(v) for v in rng.uniform(-np.pi, np.pi, (3,))],
                              "radius": float(rng.uniform(0.02, 0.05)), "length": float(rng.uniform(0.1, 0.3))})
    for _ in range(4):
        p["box"].append({"position": [float(v) for v in rng.uniform(lo, hi, (3,))],
                         "orientation_euler_xyz": [float(v) for v in rng.uniform(-np.pi, np.pi, (3,))],
                         "half_extents": [float(v) for v in rng.uniform(0.02, 0.1, (3,))]})
    env = mbm.problem_to_env(p, family)
    qrng = scenes.Rng(seed ^ 0x3C3C)
    p["start"] = [float(v) for v in scenes.sample_free("panda", env, qrng)]
    p["goals"] = [[float(v) for v in scenes.sample_free("panda", env, qrng)] for _ in range(1 + seed % 2)]
    return p


def test_mbm_problems_through_batch_planner(ctx, oracle, tmp_path):
    from prrtc_gb300 import BatchSettings, Settings, mbm
    fams = {"box": [], "table_pick": []}
    for i in range(24):
        fam = "box" if i % 2 else "table_pick"
        fams[fam].append(synthetic_problem(100 + i, fam))
    path = tmp_path / "panda_problems.json"
    path.write_text(json.dumps({"problems": fams}))
    probs = mbm.load_problems(path)
    assert len(probs) == 24
    for p in probs:
        cyl = len(fams[p.family][p.index]["cylinder"])
        if p.family == "box":        # the loader's quirk: cylinders become (r, r, r/2) cuboids
            assert len(p.env.capsules) == 0 and len(p.env.cuboids) == 4 + cyl
            r = np.float32(fams[p.family][p.index]["cylinder"][0]["radius"])
            np.testing.assert_array_equal(p.env.cuboids[0, 12:15], [r, r, r / np.float32(2.0)])
        else:
            assert len(p.env.capsules) == cyl and len(p.env.cuboids) == 4
        q = np.concatenate([p.start[None], p.goals])
        assert oracle.check("panda", p.env, q).all()
    s = Settings(max_samples=100000, max_iters=100000, num_new_configs=256, granularity=32, range=1.0, balance=0,
                 dynamic_domain=False)
    res = ctx.solve_batch("panda", [(p.env, p.start, p.goals) for p in probs], BatchSettings(s, margin=1e-5))
    solved = 0
    for p, r in zip(probs, res):
        if not r.solved:
            continue
        solved += 1
        assert any(np.array_equal(r.path[0], g) for g in p.goals)
        np.testing.assert_array_equal(r.path[-1], p.start)
        assert oracle.check_edges("panda", p.env, r.path[:-1], r.path[1:], 32).all()
    assert solved == len(probs)
