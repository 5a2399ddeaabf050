"""Synthetic workloads are deterministic and their starts/goals are free."""
import numpy as np


def test_scene_digests_stable():
    from prrtc_gb300 import scenes
    a = scenes.make_query("panda", "tabletop", 5)
    b = scenes.make_query("panda", "tabletop", 5)
    assert a.env.digest() == b.env.digest()
    np.testing.assert_array_equal(a.start, b.start)
    np.testing.assert_array_equal(a.goal, b.goal)
    assert a.env.num_obstacles == 13
    s = scenes.make_query("panda", "shelf", 5)
    assert len(s.env.cuboids) == 9 and len(s.env.capsules) == 12 and len(s.env.spheres) == 20


def test_numpy_clearance_matches_oracle(oracle):
    from prrtc_gb300 import scenes
    env = scenes.mixed_scene(4, 50)
    sc, off = (np.array(v) for v in scenes.LIMITS["fetch"])
    q = (np.random.default_rng(1).random((500, 8)) * sc + off).astype(np.float32)
    # the oracle reads the float32 model tables, numpy the float64 JSON: agree to float32 rounding
    np.testing.assert_allclose(scenes.clearance("fetch", env, q), oracle.clearance("fetch", env, q), atol=1e-6)


def test_starts_goals_free_under_oracle(oracle):
    from prrtc_gb300 import scenes
    for robot, kind in (("panda", "tabletop"), ("panda", "shelf"), ("fetch", "mixed"), ("baxter", "tabletop")):
        for seed in range(3):
            q = scenes.make_query(robot, kind, seed)
            assert oracle.check(robot, q.env, np.stack([q.start, q.goal])).all()
