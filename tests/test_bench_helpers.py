"""Host-side helpers of bench.py that shape its JSON line: the bulk rate and
tail of a launch, cost quantiles, the bytes a step uploads, and the DRAM
traffic per query read from the committed profile.  CPU only."""
import numpy as np
import pytest


def _result(solved, finish_ms, solve_ms=1.0, samples=100, status=0):
    from prrtc_gb300.api import PlannerResult
    return PlannerResult(solved=solved, finish_ns=int(finish_ms * 1e6), kernel_ns=int(solve_ms * 1e6),
                         samples=samples, status=status, start_tree_size=10, goal_tree_size=12)


def test_bulk_and_tail():
    import bench
    res = [_result(True, t) for t in range(1, 201)]                  # solved, finishing at 1 .. 200 ms
    res += [_result(False, 500.0, 499.0, 6 * 10**8, 0), _result(False, 400.0, 399.0, 10**6, 3)]
    bulk, tail = bench.bulk_and_tail(res)
    t99 = np.percentile(np.arange(1, 201) * 1e6, 99)                 # over the solved queries only
    assert abs(bulk["p99_finish_ms"] - t99 / 1e6) < 1e-9
    assert abs(bulk["queries_per_s"] - (np.arange(1, 201) * 1e6 <= t99).sum() / (t99 * 1e-9)) < 1e-6
    assert bulk["last_finish_ms"] == 200.0
    # the launch ended with the unsolved query that finished last
    assert tail["last"]["query"] == 200 and tail["last"]["solved"] is False
    assert tail["last"]["samples"] == 6 * 10**8 and tail["last"]["finish_ms"] == 500.0
    assert tail["unsolved_count"] == 2
    assert [u["status"] for u in tail["unsolved"]] == [0, 3]


def test_bulk_and_tail_without_solved_queries():
    import bench
    assert bench.bulk_and_tail([_result(False, 10.0)]) == (None, None)


def test_quantiles():
    import bench
    q = bench.quantiles(np.arange(1, 11, dtype=np.float64))
    assert q == pytest.approx({"p10": 1.9, "p50": 5.5, "p90": 9.1}, rel=1e-12)
    assert bench.quantiles([]) is None


def test_h2d_bytes_counts_packed_records():
    """Sphere 1 record, capsule 2, cuboid 4 (float4 each, as the C ABI packs
    them), the start and goal, and 24 bytes of query descriptor."""
    import bench
    from prrtc_gb300.env import Environment
    from prrtc_gb300.scenes import Query
    env = Environment(spheres=np.zeros((2, 4), np.float32), capsules=np.zeros((1, 8), np.float32),
                      z_aligned_capsules=np.zeros((1, 8), np.float32), cuboids=np.zeros((1, 15), np.float32),
                      z_aligned_cuboids=np.zeros((2, 15), np.float32))
    q = Query(env, np.zeros(7, np.float32), np.zeros(7, np.float32), 0, "test")
    assert bench.h2d_bytes([q]) == 4 * (4 * 2 + 8 * 2 + 16 * 3) + 4 * 14 + 24
    assert bench.h2d_bytes([q, q]) == 2 * bench.h2d_bytes([q])


def test_profiled_dram_bytes_per_query():
    """The bench scales the committed ncu capture of the planner kernel to a
    full launch; the summary must keep the figure it parses."""
    import bench
    v = bench.profiled_dram_bytes_per_query("panda_shelf")
    assert isinstance(v, int) and v > 0
    assert bench.profiled_dram_bytes_per_query("no_such_workload") is None
