"""Plain-form planner (prrtc_solve, the drop-in pRRTC::solve): solves, and
every returned path revalidates collision-free under the oracle checker at
the planner's granularity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def revalidate(oracle, robot, env, path, g):
    return bool(oracle.check_edges(robot, env, path[:-1], path[1:], g).all())


def c0_settings(**kw):
    from prrtc_gb300.api import Settings
    s = dict(max_samples=100000, max_iters=100000, num_new_configs=256, granularity=32, range=1.0, balance=0,
             dynamic_domain=False)
    s.update(kw)
    return Settings(**s)


@pytest.mark.parametrize("seed", range(6))
def test_tabletop_solves_and_revalidates(seed, ctx, oracle):
    from prrtc_gb300 import scenes
    q = scenes.make_query("panda", "tabletop", seed)
    s = c0_settings()
    r = ctx.solve("panda", q.start, q.goal, q.env, s)
    assert r.solved, r
    np.testing.assert_array_equal(r.path[0], q.goal)
    np.testing.assert_array_equal(r.path[-1], q.start)
    assert r.path_length == len(r.path) - 2
    assert revalidate(oracle, "panda", q.env, r.path, s.granularity)
    seg = np.linalg.norm(np.diff(r.path.astype(np.float64), axis=0), axis=1).sum()
    assert abs(seg - r.cost) < 1e-3 * max(1.0, seg)
    assert r.start_tree_size >= 1 and r.goal_tree_size >= 1 and r.kernel_ns > 0


@pytest.mark.parametrize("seed", range(3))
def test_shelf_dynamic_domain_balance2(seed, ctx, oracle):
    from prrtc_gb300 import scenes
    q = scenes.make_query("panda", "shelf", seed)
    s = c0_settings(granularity=128, balance=2, tree_ratio=1.0, dynamic_domain=True, dd_radius=4.0, dd_alpha=1e-4,
                    dd_min_radius=1.0, range=0.5)
    r = ctx.solve("panda", q.start, q.goal, q.env, s)
    assert r.solved
    assert revalidate(oracle, "panda", q.env, r.path, s.granularity)


@pytest.mark.parametrize("robot,kind", [("fetch", "mixed"), ("baxter", "tabletop"), ("sphere", "mixed")])
def test_other_robots(robot, kind, ctx, oracle):
    from prrtc_gb300 import scenes
    if robot == "sphere":
        env = scenes.mixed_scene(1, 30, (-4, -4, -4), (4, 4, 4))
        start = np.array([-4.5, -4.5, -4.5], np.float32)
        goal = np.array([4.5, 4.5, 4.5], np.float32)
        assert oracle.check("sphere", env, np.stack([start, goal])).all()
    else:
        q = scenes.make_query(robot, kind, 2, 30)
        env, start, goal = q.env, q.start, q.goal
    s = c0_settings(granularity=64, balance=1, tree_ratio=0.5)
    r = ctx.solve(robot, start, goal, env, s)
    assert r.solved
    assert revalidate(oracle, robot, env, r.path, s.granularity)


def test_multiple_goals(ctx, oracle):
    from prrtc_gb300 import scenes
    q = scenes.make_query("panda", "tabletop", 3)
    q2 = scenes.make_query("panda", "tabletop", 4)   # a second free goal in another scene
    goals = np.stack([q.goal, q2.goal]) if oracle.check("panda", q.env, q2.goal[None])[0] else q.goal[None]
    r = ctx.solve("panda", q.start, goals, q.env, c0_settings())
    assert r.solved
    assert any(np.array_equal(r.path[0], g) for g in goals)
    assert revalidate(oracle, "panda", q.env, r.path, 32)


def test_iteration_limit_and_time_budget(ctx):
    from prrtc_gb300 import scenes
    q = scenes.make_query("panda", "shelf", 0)
    r = ctx.solve("panda", q.start, q.goal, q.env, c0_settings(max_iters=1, num_new_configs=4))
    assert not r.solved and r.status == 0 and r.iters == -1
    ctx.set_time_budget(1)          # 1 ns: the first check ends the search
    try:
        r = ctx.solve("panda", q.start, q.goal, q.env, c0_settings(num_new_configs=4))
        assert not r.solved and r.status == 3
    finally:
        ctx.set_time_budget(0)
