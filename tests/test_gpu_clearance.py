"""Differentiable clearance on the GPU (prrtc_path_cost_grad,
prrtc_smooth_paths) against the oracle.

Inputs are planned paths: Panda tabletop and shelf, Baxter tabletop and Fetch
mixed-clutter queries solved by the batched planner, resampled to 64 float32 waypoints.  The
library's adjoint must match the oracle's float64 adjoint to 1e-4 (relative,
per waypoint, plus 1e-9 absolute for waypoints whose gradient vanishes) and the
central finite differences of the library's own cost at h = 1e-3 rad within
the truncation bound the hinge allows.  Every smoothed path the library
accepts must pass the oracle's checker at 128 points per edge, and every path
it rejects must come back bit for bit as it went in.  A torch.autograd.Function
over the C ABI (this file only) drives the same descent from torch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN = 0.02
W = 64


def floored_rel(a, b):
    a, b = a.reshape(-1, a.shape[-1]), b.reshape(-1, b.shape[-1])
    return np.linalg.norm(a - b, axis=1) / (np.linalg.norm(b, axis=1) + 1e-6)


@pytest.fixture(scope="module")
def planned(ctx):
    """{robot: (envs, paths [P, W, dof])} from batched-planner solutions."""
    from prrtc_gb300 import BatchSettings, Settings, paths, scenes
    out = {}
    plan = {
        "panda": ([scenes.make_query("panda", "tabletop", i) for i in range(48)] +
                  [scenes.make_query("panda", "shelf", i) for i in range(32)],
                  Settings(granularity=128, balance=2, tree_ratio=1.0, dynamic_domain=True, range=0.5)),
        "baxter": ([scenes.make_query("baxter", "tabletop", i, z_offset=0.3) for i in range(24)],
                   Settings(granularity=128, balance=1, tree_ratio=0.5)),
        # Fetch: the robot with a prismatic joint (torso lift), mixed clutter
        "fetch": ([scenes.make_query("fetch", "mixed", 300 + i, 30) for i in range(32)], Settings(granularity=64)),
    }
    for robot, (qs, s) in plan.items():
        res = ctx.solve_batch(robot, qs, BatchSettings(s, margin=1e-5), path_capacity=4096)
        envs, ps = [], []
        for q, r in zip(qs, res):
            if not r.solved:
                continue
            p = paths.resample(paths.start_first(r.path), W)
            if p is not None:
                envs.append(q.env)
                ps.append(p)
        assert len(ps) >= len(qs) // 2, (robot, len(ps))
        out[robot] = (envs, np.stack(ps))
    return out


@pytest.mark.parametrize("robot", ["panda", "baxter", "fetch"])
def test_adjoint_matches_fp64(ctx, oracle, planned, robot):
    envs, P = planned[robot]
    cost, grad = ctx.path_cost_grad(robot, envs, P, MARGIN)
    c64 = np.empty(cost.shape)
    g64 = np.empty(grad.shape)
    for i, e in enumerate(envs):
        c64[i], g64[i] = oracle.cost_grad(robot, e, P[i].astype(np.float64), MARGIN)
    assert (c64 > 0).any()
    np.testing.assert_allclose(cost, c64, rtol=1e-4, atol=1e-9)
    # per waypoint: relative 1e-4, plus 1e-9 absolute (the float32 resolution of
    # gradient entries of order 1e-2; a waypoint whose true gradient is ~1e-6
    # is otherwise judged on rounding alone)
    err = np.linalg.norm((grad - g64).reshape(-1, grad.shape[-1]), axis=1)
    ref = np.linalg.norm(g64.reshape(-1, grad.shape[-1]), axis=1)
    worst = np.max(err - 1e-4 * ref)
    assert worst <= 1e-9, (worst, np.median(floored_rel(grad, g64)))
    assert np.linalg.norm(grad - g64) / np.linalg.norm(g64) <= 1e-4


@pytest.mark.parametrize("robot", ["panda", "baxter"])
def test_adjoint_matches_finite_differences(ctx, planned, robot):
    """Central differences of the library's cost, h = 1e-3 rad."""
    envs, P = planned[robot]
    _, g_all = ctx.path_cost_grad(robot, envs, P, MARGIN)
    # the 16 paths with the most waypoints inside the margin (planner output varies run to run)
    idx = np.argsort(-(np.linalg.norm(g_all, axis=-1) > 1e-4).sum(1), kind="stable")[:16]
    P = P[idx]
    envs = [envs[i] for i in idx]
    _, grad = ctx.path_cost_grad(robot, envs, P, MARGIN)
    D = P.shape[2]
    fd = np.zeros_like(grad, dtype=np.float64)
    h = 1e-3
    for d in range(D):
        plus, minus = P.copy(), P.copy()
        plus[..., d] += np.float32(h)
        minus[..., d] -= np.float32(h)
        step = (plus[..., d].astype(np.float64) - minus[..., d].astype(np.float64))   # the float32 step taken
        cp, _ = ctx.path_cost_grad(robot, envs, plus, MARGIN)
        cm, _ = ctx.path_cost_grad(robot, envs, minus, MARGIN)
        fd[..., d] = (cp.astype(np.float64) - cm.astype(np.float64)) / step
    active = np.linalg.norm(grad, axis=-1).reshape(-1) > 1e-4
    rel = floored_rel(grad, fd)[active]
    assert active.sum() >= 8
    assert np.median(rel) <= 1e-3, np.median(rel)
    assert np.linalg.norm((grad - fd).reshape(-1, D)[active]) / np.linalg.norm(fd.reshape(-1, D)[active]) <= 2e-2


def test_device_pointers_match_host(ctx, planned):
    torch = pytest.importorskip("torch")
    envs, P = planned["panda"]
    c_h, g_h = ctx.path_cost_grad("panda", envs, P, MARGIN)
    c_d, g_d = ctx.path_cost_grad("panda", envs, torch.from_numpy(P).cuda(), MARGIN)
    np.testing.assert_array_equal(c_d.cpu().numpy(), c_h)
    np.testing.assert_array_equal(g_d.cpu().numpy(), g_h)


@pytest.mark.parametrize("robot", ["panda", "baxter"])
def test_smooth_paths_judged_by_checker(ctx, oracle, planned, robot):
    from prrtc_gb300 import SmoothSettings, paths
    envs, P = planned[robot]
    s = SmoothSettings()
    assert (s.steps, s.granularity) == (50, 128) and abs(s.margin - MARGIN) < 1e-9
    out, acc, cb, ca = ctx.smooth_paths(robot, envs, P, s)
    c0, _ = ctx.path_cost_grad(robot, envs, P, MARGIN)
    np.testing.assert_allclose(cb, c0.sum(1), rtol=1e-5)
    c1, _ = ctx.path_cost_grad(robot, envs, out, MARGIN)
    for i, e in enumerate(envs):
        if acc[i]:
            assert oracle.check_edges(robot, e, out[i, :-1], out[i, 1:], 128).all(), i
            np.testing.assert_array_equal(out[i, 0], P[i, 0])
            np.testing.assert_array_equal(out[i, -1], P[i, -1])
            np.testing.assert_allclose(ca[i], c1[i].sum(), rtol=1e-5, atol=1e-9)
        else:
            np.testing.assert_array_equal(out[i], P[i])
    assert acc.mean() >= 0.5, acc.mean()
    a = acc.astype(bool)
    assert ca[a].sum() < cb[a].sum()                                 # clearance improved
    assert paths.length(out[a]).sum() < paths.length(P[a]).sum()     # and the paths got shorter


def test_smooth_in_place_on_device_matches_host(ctx, planned):
    torch = pytest.importorskip("torch")
    envs, P = planned["panda"]
    out_h, acc_h, cb_h, ca_h = ctx.smooth_paths("panda", envs, P)
    t = torch.from_numpy(P).cuda()
    out_d, acc_d, cb_d, ca_d = ctx.smooth_paths("panda", envs, t)
    assert out_d.data_ptr() == t.data_ptr()
    np.testing.assert_array_equal(out_d.cpu().numpy(), out_h)
    np.testing.assert_array_equal(acc_d.cpu().numpy(), acc_h)
    np.testing.assert_array_equal(ca_d.cpu().numpy(), ca_h)


def test_bad_arguments(ctx, planned):
    from prrtc_gb300 import PrrtcError, SmoothSettings
    envs, P = planned["panda"]
    big = np.zeros((1, 257, 7), np.float32)
    with pytest.raises(PrrtcError):
        ctx.smooth_paths("panda", envs[:1], big)
    with pytest.raises(PrrtcError):
        ctx.smooth_paths("panda", envs[:1], P[:1], SmoothSettings(granularity=0))
    with pytest.raises(PrrtcError):
        ctx.path_cost_grad("panda", envs[:1], P[:1], -1.0)


def clearance_cost(ctx, robot, envs):
    """torch.autograd.Function over prrtc_path_cost_grad (test harness only):
    forward returns the per-waypoint cost, backward the library's adjoint."""
    import torch

    class ClearanceCost(torch.autograd.Function):
        @staticmethod
        def forward(fctx, q):
            cost, grad = ctx.path_cost_grad(robot, envs, q.detach().contiguous(), MARGIN)
            fctx.save_for_backward(grad)
            return cost

        @staticmethod
        def backward(fctx, g_out):
            (grad,) = fctx.saved_tensors
            return grad * g_out.unsqueeze(-1)

    return ClearanceCost.apply


def test_autograd_shim_descent(ctx, oracle, planned):
    torch = pytest.importorskip("torch")
    envs, P = planned["panda"]
    envs, P = envs[:32], P[:32]
    cost_fn = clearance_cost(ctx, "panda", envs)
    q = torch.from_numpy(P).cuda().requires_grad_(True)
    cost_fn(q).sum().backward()
    g64 = np.stack([oracle.cost_grad("panda", e, P[i].astype(np.float64), MARGIN)[1] for i, e in enumerate(envs)])
    g = q.grad.cpu().numpy()
    assert np.max(np.linalg.norm(g - g64, axis=-1) - 1e-4 * np.linalg.norm(g64, axis=-1)) <= 1e-9
    # the library's smoothing iteration (without the joint-limit clamp),
    # driven from torch: d/dx of 1/2 sum |x_{w+1} - x_w|^2 is the path Laplacian
    x = torch.from_numpy(P).cuda()
    for _ in range(50):
        x = x.detach().requires_grad_(True)
        loss = 100.0 * cost_fn(x).sum() + 0.5 * (x[:, 1:] - x[:, :-1]).pow(2).sum()
        loss.backward()
        with torch.no_grad():
            step = x.grad.clone()
            step[:, 0] = 0
            step[:, -1] = 0
            x = x - 0.05 * step
    out = x.detach().cpu().numpy()
    assert np.isfinite(out).all()
    ok = [oracle.check_edges("panda", e, out[i, :-1], out[i, 1:], 128).all() for i, e in enumerate(envs)]
    assert np.mean(ok) >= 0.5
    assert cost_fn(x.detach()).sum().item() < cost_fn(torch.from_numpy(P).cuda()).sum().item()


def test_shortcuts_alone(ctx, oracle, planned):
    """Shortcut attempts only (no gradient steps): every accepted path is
    clean under the oracle at 128 points per edge, keeps its end points and
    is no longer than before; most paths get shorter."""
    from prrtc_gb300 import SmoothSettings, paths
    envs, P = planned["panda"]
    out, acc, _, _ = ctx.smooth_paths("panda", envs, P, SmoothSettings(steps=0, shortcut_rounds=64))
    a = acc.astype(bool)
    assert a.mean() >= 0.5, a.mean()
    for i in np.flatnonzero(a):
        assert oracle.check_edges("panda", envs[i], out[i, :-1], out[i, 1:], 128).all(), i
        np.testing.assert_array_equal(out[i, [0, -1]], P[i, [0, -1]])
    before, after = paths.length(P[a]), paths.length(out[a])
    assert (after <= before * (1 + 1e-5)).all()
    assert (after < before * 0.99).mean() >= 0.5
