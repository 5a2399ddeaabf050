"""pRRTC's own GPU planner (rrtc<Robot>, run from the cubin oracle/_ref holds)
beside the drop-in plain form on the same GB300, under settings for which
every write of the reference kernel provably stays in bounds
(pyoracle.RefPlanner.safe_rows: dynamic domain off, few lanes and
iterations; see its docstring).  Panda tabletop queries (the C0 scene kind),
range 1.0, granularity 32, balance 0.

* One lane, 46 iterations: both planners are deterministic and draw the
  same Halton points (lane 0's bases are the unshuffled primes), so their
  results are compared query by query.
* Four lanes, 10 iterations: success rate and p50 kernel time side by side.
  Four concurrent lanes race on the trees in both planners, so which
  queries get solved within 40 samples varies run to run; the success counts
  must agree within three standard deviations of their difference
  (binomial, 64 queries).
Every returned path of either planner is revalidated by the oracle."""
import statistics

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def settings(lanes, iters):
    from prrtc_gb300 import Settings
    return Settings(max_samples=714, max_iters=iters, num_new_configs=lanes, granularity=32, range=1.0, balance=0,
                    dynamic_domain=False)


@pytest.fixture(scope="module")
def ref():
    from pyoracle import RefPlanner
    if not RefPlanner.available():
        pytest.skip("pRRTC's planner cubin not built (needs a pRRTC checkout at build time)")
    return RefPlanner("panda")


def run_both(ctx, ref, oracle, s, n, seed0):
    from prrtc_gb300 import scenes
    ctx.set_planning_margin(0.0)
    ctx.set_time_budget(0)
    rows = []
    for i in range(n):
        q = scenes.make_query("panda", "tabletop", seed0 + i)
        a = ref.solve(q.start, q.goal, q.env, s)
        b = ctx.solve("panda", q.start, q.goal, q.env, s)
        for p in ([a["path"]] if a["solved"] else []) + ([b.path] if b.solved else []):
            np.testing.assert_array_equal(p[0], q.goal)
            np.testing.assert_array_equal(p[-1], q.start)
            assert oracle.check_edges("panda", q.env, p[:-1], p[1:], s.granularity).all()
        rows.append((a, b))
    return rows


def test_single_lane_runs_match_reference(ctx, ref, oracle):
    s = settings(1, 46)
    rows = run_both(ctx, ref, oracle, s, 32, 0)
    same_flag = sum(a["solved"] == b.solved for a, b in rows)
    both = [(a, b) for a, b in rows if a["solved"] and b.solved]
    same_path = sum(a["path"].shape == b.path.shape and np.array_equal(a["path"], b.path) for a, b in both)
    same_trees = sum(a["start_tree_size"] == b.start_tree_size and a["goal_tree_size"] == b.goal_tree_size
                     for a, b in rows)
    print(f"1 lane x 46 iterations, 32 queries: solved flags equal {same_flag}/32, identical paths "
          f"{same_path}/{len(both)}, identical tree sizes {same_trees}/32; reference solved "
          f"{sum(a['solved'] for a, _ in rows)}, plain form solved {sum(b.solved for _, b in rows)}")
    assert same_flag >= 30 and same_path >= 0.75 * len(both)


def test_p50_beside_reference(ctx, ref, oracle):
    s = settings(4, 10)
    ref.solve(np.zeros(7), np.zeros((1, 7)), __import__("prrtc_gb300").scenes.tabletop_scene(0), s)   # warm-up
    rows = run_both(ctx, ref, oracle, s, 64, 100)
    ra = [a["kernel_ms"] for a, _ in rows if a["solved"]]
    rb = [b.kernel_ns / 1e6 for _, b in rows if b.solved]
    sa, sb = len(ra), len(rb)
    print(f"4 lanes x 10 iterations, 64 queries: pRRTC solved {sa} (p50 kernel {statistics.median(ra):.3f} ms), "
          f"plain form solved {sb} (p50 kernel {statistics.median(rb):.3f} ms)")
    p = (sa + sb) / 128
    assert abs(sa - sb) <= max(3.0, 3 * (2 * 64 * p * (1 - p)) ** 0.5), (sa, sb)
