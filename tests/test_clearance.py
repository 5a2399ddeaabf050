"""Differentiable clearance on the CPU: the float64 adjoint of the oracle
against central finite differences, the cost's exact relation to the
clearance, an analytic box case, and the path resampler."""
import numpy as np
import pytest

MARGIN = 0.02
CASES = [("panda", "tabletop"), ("panda", "shelf"), ("fetch", "mixed"), ("baxter", "tabletop")]


def scene(kind, seed=1):
    from prrtc_gb300 import scenes
    if kind == "tabletop":
        return scenes.tabletop_scene(seed)
    if kind == "shelf":
        return scenes.shelf_scene(seed)
    return scenes.mixed_scene(seed, 40)


def near_contact_free(oracle, robot, env, n, seed=3):
    """Collision-free configurations with some leaf test inside the margin:
    what waypoints of planned paths look like."""
    from prrtc_gb300 import scenes
    q = scenes._uniform_configs(robot, scenes.Rng(seed), 30000).astype(np.float32)
    q = q[np.asarray(oracle.check(robot, env, q)) == 1].astype(np.float64)
    cost, _ = oracle.cost_grad(robot, env, q, MARGIN)
    return q[cost > 0][:n]


def central_fd(oracle, robot, env, q, h):
    D = q.shape[1]
    fd = np.zeros_like(q)
    for d in range(D):
        e = np.zeros(D)
        e[d] = h
        fd[:, d] = (oracle.cost_grad(robot, env, q + e, MARGIN)[0] - oracle.cost_grad(robot, env, q - e, MARGIN)[0]) / (2 * h)
    return fd


def floored_rel(a, b):
    """Per-row |a - b| / (|b| + 1e-6): rows whose gradient vanishes (a cost
    made only of rigidly attached sphere pairs) compare absolutely."""
    return np.linalg.norm(a - b, axis=1) / (np.linalg.norm(b, axis=1) + 1e-6)


@pytest.mark.parametrize("robot,kind", CASES)
def test_oracle_adjoint_matches_finite_differences(oracle, robot, kind):
    env = scene(kind)
    q = near_contact_free(oracle, robot, env, 200)
    assert len(q) >= 100
    _, g = oracle.cost_grad(robot, env, q, MARGIN)
    rel = floored_rel(central_fd(oracle, robot, env, q, 1e-6), g)
    assert rel.max() <= 1e-4, (rel.max(), np.median(rel))


def test_fd_at_1e3_truncation_is_bounded(oracle):
    """At h = 1e-3 rad central differences carry truncation error where a
    hinge term switches on or off within +-h; most waypoints still agree to
    1e-4 and the whole-set error stays small."""
    env = scene("tabletop")
    q = near_contact_free(oracle, "panda", env, 400)
    _, g = oracle.cost_grad("panda", env, q, MARGIN)
    fd = central_fd(oracle, "panda", env, q, 1e-3)
    rel = floored_rel(fd, g)
    assert (rel <= 1e-4).mean() >= 0.9
    assert np.linalg.norm(fd - g) / np.linalg.norm(g) <= 5e-3


@pytest.mark.parametrize("robot,kind", CASES)
def test_cost_positive_exactly_inside_margin(oracle, robot, kind):
    """C(q) > 0 exactly when the float64 clearance over the same leaf tests is
    below the margin (inside a box the true distance is below the reference's
    flat one, so both are below the margin there)."""
    from prrtc_gb300 import scenes
    env = scene(kind)
    q = scenes._uniform_configs(robot, scenes.Rng(11), 3000).astype(np.float32)
    clear = oracle.clearance(robot, env, q)
    cost, _ = oracle.cost_grad(robot, env, q.astype(np.float64), MARGIN)
    sure = np.abs(clear - MARGIN) > 1e-9
    np.testing.assert_array_equal((cost > 0)[sure], (clear < MARGIN)[sure])
    assert (cost > 0).any()


def test_box_interior_gradient(oracle):
    """The toy sphere robot (radius 1) inside a box: the gradient follows the
    nearest face, with the analytic value -(m - (q_face - r))."""
    from prrtc_gb300.env import Environment, cuboid_row
    env = Environment(cuboids=np.array([cuboid_row((0.0, 0.0, 0.0), (3.0, 4.0, 5.0))], np.float32))
    q = np.array([[2.5, 0.3, -0.2], [0.1, -3.2, 0.0], [0.0, 0.5, 4.6]])
    c = oracle.fk_spheres("sphere", q)[:, 0, :3]
    np.testing.assert_allclose(c, q, atol=1e-12)   # the toy robot's sphere sits at q
    cost, g = oracle.cost_grad("sphere", env, q, MARGIN)
    depth = np.array([3.0 - 2.5, 4.0 - 3.2, 5.0 - 4.6])     # distance to the nearest face
    phi = MARGIN + depth + 1.0
    np.testing.assert_allclose(cost, 0.5 * phi ** 2, rtol=1e-12)
    want = np.zeros((3, 3))
    want[0, 0], want[1, 1], want[2, 2] = -phi[0], phi[1], -phi[2]
    np.testing.assert_allclose(g, want, rtol=1e-12, atol=1e-12)


def test_resample_keeps_vertices():
    from prrtc_gb300 import paths
    rng = np.random.default_rng(0)
    p = rng.normal(size=(9, 7)).astype(np.float32)
    r = paths.resample(p, 64)
    assert r.shape == (64, 7) and r.dtype == np.float32
    idx = [int(np.argmin(np.abs(r - v).sum(1))) for v in p]
    assert idx == sorted(idx) and idx[0] == 0 and idx[-1] == 63
    np.testing.assert_array_equal(r[idx], p)
    assert abs(paths.length(r) - paths.length(p)) < 1e-4 * paths.length(p)
    assert paths.resample(rng.normal(size=(65, 7)), 64) is None
    assert paths.start_first(p)[0].tolist() == p[-1].tolist()
