"""Goal regions (prrtc_sample_goals): configurations whose hand sphere lies in
a shelf cell, checked against the oracle (float64 kinematics, the reference
checker's verdict), deterministic for fixed arguments, and usable as a goal
set by the batched planner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_goal_region_in_shelf_cell(ctx, oracle):
    from prrtc_gb300 import BatchSettings, Settings, scenes
    q = scenes.make_query("panda", "shelf", 3)
    hand = scenes.hand_sphere("panda")
    lo, hi = scenes.shelf_cells()[4]          # the middle cell
    goals = ctx.sample_goals("panda", q.env, hand, lo, hi, max_goals=8, tries=1 << 21, seed=7)
    assert 1 <= len(goals) <= 8
    c = oracle.fk_spheres("panda", goals.astype(np.float64))[:, hand, :3]
    assert ((c >= lo - 1e-5) & (c <= hi + 1e-5)).all()
    assert np.asarray(oracle.check("panda", q.env, goals)).all()
    again = ctx.sample_goals("panda", q.env, hand, lo, hi, max_goals=8, tries=1 << 21, seed=7)
    np.testing.assert_array_equal(goals, again)
    other = ctx.sample_goals("panda", q.env, hand, lo, hi, max_goals=8, tries=1 << 21, seed=8)
    assert not np.array_equal(goals[:1], other[:1])

    s = Settings(granularity=128, balance=2, tree_ratio=1.0, dynamic_domain=True)
    [r] = ctx.solve_batch("panda", [(q.env, q.start, goals)], BatchSettings(s, margin=1e-5))
    assert r.solved
    assert any(np.array_equal(r.path[0], g) for g in goals)   # the path starts at one of the goals
    np.testing.assert_array_equal(r.path[-1], q.start)
    assert oracle.check_edges("panda", q.env, r.path[:-1], r.path[1:], 128).all()


def test_goal_region_bad_arguments(ctx):
    from prrtc_gb300 import PrrtcError, scenes
    q = scenes.make_query("panda", "shelf", 3)
    with pytest.raises(PrrtcError):
        ctx.sample_goals("panda", q.env, 10_000, (0, 0, 0), (1, 1, 1))
    empty = ctx.sample_goals("panda", q.env, 0, (5, 5, 5), (6, 6, 6), tries=4096)   # an unreachable box
    assert empty.shape == (0, 7)
