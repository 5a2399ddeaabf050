"""The oracle against the reference: golden fixtures made by pRRTC's own
checker, live comparison when the reference is present, MBM known answers,
and the planner restatement's own consistency (CPU)."""
import numpy as np
import pytest

from conftest import REFERENCE, golden_cases, load_golden


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_matches_reference_verdicts(case, oracle):
    robot = case.split("_")[0]
    env, z = load_golden(case)
    free, margin = oracle.check(robot, env, z["q"], margin=True)
    bad = np.flatnonzero(free != z["free_ref"])
    # disagreements may only sit within 1e-5 m of contact
    assert np.all(margin[bad] < 1e-5), (len(bad), margin[bad].min() if len(bad) else None)
    assert len(bad) <= (margin < 1e-5).sum()
    np.testing.assert_allclose(margin, z["margin"], rtol=0, atol=1e-9)


@pytest.mark.skipif(not (REFERENCE / "src/planning/utils.cuh").exists(), reason="reference checkout absent")
@pytest.mark.parametrize("robot", ["panda", "fetch", "baxter", "sphere"])
def test_oracle_matches_reference_live(robot, oracle):
    from pyoracle import RefLib, build
    if not RefLib.available():
        build(ref=True)
    R = RefLib()
    from prrtc_gb300 import scenes
    env = scenes.mixed_scene(99, 60, n_zaligned=12) if robot != "sphere" else scenes.mixed_scene(
        99, 60, (-4, -4, -4), (4, 4, 4), n_zaligned=20)
    sc, off = (np.array(v) for v in scenes.LIMITS[robot])
    q = (np.random.default_rng(3).random((100000, len(sc))) * sc + off).astype(np.float32)
    a = R.check(robot, env, q)
    b, m = oracle.check(robot, env, q, margin=True)
    bad = np.flatnonzero(a != b)
    assert np.all(m[bad] < 1e-5)


@pytest.mark.parametrize("robot", ["sphere", "panda", "fetch", "baxter"])
def test_zaligned_fixtures_decide_verdicts(robot, oracle):
    """Each robot has a golden fixture holding z-aligned capsules and
    z-aligned cuboids whose verdicts depend on them: dropping either type
    frees some configurations (utils.cuh:134-148,178-197 really run)."""
    from prrtc_gb300.env import Environment
    flips_c = flips_b = 0
    for case in golden_cases():
        if not case.startswith(robot + "_z"):
            continue
        env, z = load_golden(case)
        assert len(env.z_aligned_capsules) and len(env.z_aligned_cuboids)
        q = z["q"]
        full = oracle.check(robot, env, q)
        np.testing.assert_array_equal(full[z["margin"] > 1e-5], z["free_ref"][z["margin"] > 1e-5])
        no_c = Environment(spheres=env.spheres, capsules=env.capsules, cuboids=env.cuboids,
                           z_aligned_cuboids=env.z_aligned_cuboids)
        no_b = Environment(spheres=env.spheres, capsules=env.capsules, cuboids=env.cuboids,
                           z_aligned_capsules=env.z_aligned_capsules)
        flips_c += int((oracle.check(robot, no_c, q) != full).sum())
        flips_b += int((oracle.check(robot, no_b, q) != full).sum())
    assert flips_c > 0 and flips_b > 0, (flips_c, flips_b)


MBM = [("panda", REFERENCE / "scripts/panda_problems.json"), ("fetch", REFERENCE / "scripts/fetch_problems.json")]


@pytest.mark.parametrize("robot,path", MBM)
def test_mbm_starts_and_goals_are_free(robot, path, oracle):
    """Known answers: every valid MotionBenchMaker start and goal is free
    under the reference checker (read from the reference checkout at test
    time; no problem data is stored in this repository)."""
    if not path.exists():
        pytest.skip("reference checkout absent")
    from prrtc_gb300.mbm import load_problems
    probs = load_problems(path)
    assert len(probs) > 600
    flagged = 0
    for p in probs:
        q = np.concatenate([p.start[None], p.goals])
        flagged += int((oracle.check(robot, p.env, q) == 0).sum())
    assert flagged == 0


def test_edges_match_pointwise(oracle):
    from prrtc_gb300 import scenes
    env, z = load_golden("panda_tabletop")
    q = z["q"]
    a, b = q[:300], q[300:600]
    g = 16
    got = oracle.check_edges("panda", env, a, b, g)
    step = (b - a) / np.float32(g)
    pts = np.stack([a + np.float32(k) * step for k in range(1, g + 1)], 1).reshape(-1, 7).astype(np.float32)
    pf = oracle.check("panda", env, pts).reshape(300, g)
    np.testing.assert_array_equal(got, pf.all(1).astype(np.uint8))


def test_oracle_planner_paths_revalidate(oracle):
    from prrtc_gb300 import scenes
    from prrtc_gb300.api import Settings
    s = Settings(max_samples=20000, max_iters=2000, num_new_configs=32, granularity=16, range=1.0, balance=0,
                 dynamic_domain=False)
    solved = 0
    for seed in range(4):
        q = scenes.make_query("panda", "tabletop", seed)
        r, path = oracle.solve("panda", q.start, q.goal, q.env, s)
        if not r.solved:
            continue
        solved += 1
        np.testing.assert_array_equal(path[0], q.goal)
        np.testing.assert_array_equal(path[-1], q.start)
        assert oracle.check_edges("panda", q.env, path[:-1], path[1:], s.granularity).all()
    assert solved >= 3
