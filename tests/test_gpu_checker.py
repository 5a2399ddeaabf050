"""GPU collision checker parity (validate_configs / validate_edges /
fk_spheres through the C ABI) against the reference's verdicts and the oracle.

Bar: every verdict equal, except configurations whose float64 near-contact
measure (min |signed distance| over the checker's tests) is below 1e-5 m;
those are counted and reported.  FK sphere centres within 1e-5 m of float64 FK.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu
NEAR = 1e-5


@pytest.mark.parametrize("case", golden_cases())
def test_checker_matches_reference_golden(case, ctx, oracle):
    robot = case.split("_")[0]
    env, z = load_golden(case)
    got = ctx.validate_configs(robot, env, z["q"])
    bad = np.flatnonzero(got != z["free_ref"])
    print(f"{case}: {len(z['q'])} configs, mismatches {len(bad)}, near-contact {(z['margin'] < NEAR).sum()}")
    assert np.all(z["margin"][bad] < NEAR)


SCENES = [("panda", "tabletop", 0), ("panda", "shelf", 1), ("fetch", "mixed", 2), ("baxter", "shelf", 3),
          ("baxter", "mixed", 4)]


def scene(robot, kind, seed):
    """Every scene also holds z-aligned capsules and z-aligned cuboids
    (tabletop 8, shelf 6, mixed 12), so all five primitive tests run."""
    from prrtc_gb300 import scenes
    if kind == "mixed":
        return scenes.mixed_scene(seed, 60, n_zaligned=12)
    if kind == "shelf":
        return scenes.shelf_scene(seed, 0.3 if robot == "baxter" else 0.0, n_zaligned=6)
    return scenes.tabletop_scene(seed, n_zaligned=8)


def million(robot, seed):
    from prrtc_gb300 import scenes
    sc, off = (np.array(v) for v in scenes.LIMITS[robot])
    rng = np.random.default_rng(100 + seed)
    return (rng.random((1_000_000, len(sc))) * sc + off).astype(np.float32)


@pytest.mark.parametrize("robot,kind,seed", SCENES)
def test_checker_million_configs(robot, kind, seed, ctx, oracle):
    env = scene(robot, kind, seed)
    q = million(robot, seed)
    got = ctx.validate_configs(robot, env, q)
    ref, margin = oracle.check(robot, env, q, margin=True)
    bad = np.flatnonzero(got != ref)
    near = int((margin < NEAR).sum())
    print(f"{robot}/{kind}: 1e6 configs, free {ref.mean():.3f}, mismatches {len(bad)}, near-contact bucket {near}")
    assert np.all(margin[bad] < NEAR)


@pytest.mark.parametrize("robot,kind,seed", SCENES + [("sphere", "mixed", 5)])
def test_checker_matches_reference_gpu_checker(robot, kind, seed, ctx, oracle):
    """Verdicts against pRRTC's own GPU checker (fkcc<Robot>, utils.cuh:326-327,
    compiled for sm_103a from the reference sources into oracle/_ref and
    loaded as a cubin) on 10^6 seeded configurations per robot, in scenes
    with every primitive type.  Disagreements may only lie in the
    near-contact bucket (float64 margin < 1e-5 m), which is counted."""
    from pyoracle import RefGpuChecker
    if not RefGpuChecker.available(robot):
        pytest.skip("reference GPU checker not built (needs a pRRTC checkout at build time)")
    from prrtc_gb300 import scenes
    env = scene(robot, kind, seed) if robot != "sphere" else scenes.mixed_scene(
        seed, 60, (-4, -4, -4), (4, 4, 4), n_zaligned=20)
    q = million(robot, seed)
    ref = RefGpuChecker(robot).check(env, q)
    got = ctx.validate_configs(robot, env, q)
    _, margin = oracle.check(robot, env, q, margin=True)
    bad = np.flatnonzero(got != ref)
    near = int((margin < NEAR).sum())
    print(f"{robot}/{kind} vs pRRTC GPU checker: 1e6 configs, free {ref.mean():.4f}, mismatches {len(bad)}, "
          f"near-contact bucket {near}")
    assert np.all(margin[bad] < NEAR)


def test_checker_faster_than_reference_gpu_checker(ctx):
    """Device time of prrtc_validate_configs against pRRTC's own checker
    kernel (fkcc<Robot>, utils.cuh:326-327, one configuration per thread in
    128-thread blocks, as pRRTC.cu:441,529 check interpolated points) on the
    same 2^20 configurations: uniformly random, then collision-free (the
    random set's free configurations repeated).  L2 is flushed before every
    launch; median of 5 after one warm-up.  Both kernels see the same inputs
    already on the device; the table prints with `pytest -s`.  The verdicts
    are counted against each other (parity proper is the test above) and
    the library's kernel must be the faster in every case."""
    import statistics

    import torch
    from pyoracle import RefGpuChecker
    from prrtc_gb300 import scenes
    if not all(RefGpuChecker.available(r) for r in ("panda", "fetch", "baxter")):
        pytest.skip("reference GPU checker not built (needs a pRRTC checkout at build time)")
    n = 1 << 20
    cases = [("panda", "tabletop 0", scenes.tabletop_scene(0)), ("panda", "shelf 1", scenes.shelf_scene(1))]
    cases += [(r, f"{k} {s}, all types", scene(r, k, s)) for r, k, s in SCENES]
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")

    def timed(fn):
        ms = []
        for _ in range(6):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ms.append(fn())
        return statistics.median(ms[1:])

    def ref_ms(run):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        run()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    rows = []
    for robot, label, env in cases:
        ref = RefGpuChecker(robot)
        e = ctx.upload_env(env)
        sc, off = (np.array(v) for v in scenes.LIMITS[robot])
        rnd = (np.random.default_rng(7).random((n, len(sc))) * sc + off).astype(np.float32)
        qr = torch.from_numpy(rnd).cuda()
        free = ctx.validate_configs(robot, e, qr).cpu().numpy().astype(bool)
        qf = torch.from_numpy(np.ascontiguousarray(np.resize(rnd[free], (n, len(sc))))).cuda()
        for kind, q in (("random", qr), ("free", qf)):
            run, out = ref.prepare(env, q)
            t_ref = timed(lambda: ref_ms(run))
            got = []

            def ours():
                got.append(ctx.validate_configs(robot, e, q))
                torch.cuda.synchronize()
                return ctx.last_kernel_ns() / 1e6
            t_ours = timed(ours)
            mism = int((got[-1] != out).sum().item())
            rows.append((robot, label, kind, t_ref, t_ours, mism))
    print("\nrobot   scene                    configs  pRRTC fkcc ms  library ms  speed-up  mismatches")
    for robot, label, kind, t_ref, t_ours, mism in rows:
        print(f"{robot:7s} {label:24s} {kind:7s}  {t_ref:13.3f}  {t_ours:10.3f}  {t_ref / t_ours:7.2f}x  {mism}")
    for robot, label, kind, t_ref, t_ours, mism in rows:
        assert mism <= n // 100000, (robot, label, kind, mism)
        assert t_ours < t_ref, (robot, label, kind, t_ours, t_ref)


@pytest.mark.parametrize("case", golden_cases())
def test_fk_spheres_match_fp64(case, ctx, oracle):
    robot = case.split("_")[0]
    env, z = load_golden(case)
    got = ctx.fk_spheres(robot, z["q"])
    ref = oracle.fk_spheres(robot, z["q"].astype(np.float64))
    assert np.abs(got[..., :3] - ref[..., :3]).max() < 1e-5
    np.testing.assert_array_equal(got[..., 3], ref[..., 3].astype(np.float32))
    # against the reference's own generated FK evaluated in float64
    fk = ctx.fk_spheres(robot, z["fk_q"])
    assert np.abs(fk[..., :3] - z["fk_centres"]).max() < 1e-5


@pytest.mark.parametrize("robot,kind,seed", SCENES[:3])
@pytest.mark.parametrize("g", [1, 32, 128])
def test_edges_match_oracle(robot, kind, seed, g, ctx, oracle):
    from prrtc_gb300 import scenes
    env = scene(robot, kind, seed)
    sc, off = (np.array(v) for v in scenes.LIMITS[robot])
    rng = np.random.default_rng(7 + seed)
    a = (rng.random((3000, len(sc))) * sc + off).astype(np.float32)
    b = (a + rng.normal(0, 0.3, a.shape)).astype(np.float32)
    got = ctx.validate_edges(robot, env, a, b, g)
    ref = oracle.check_edges(robot, env, a, b, g)
    bad = np.flatnonzero(got != ref)
    for i in bad:   # a disagreement needs a near-contact point on that edge
        step = (b[i] - a[i]) / np.float32(g)
        pts = np.stack([a[i] + np.float32(k) * step for k in range(1, g + 1)]).astype(np.float32)
        _, m = oracle.check(robot, env, pts, margin=True)
        assert m.min() < NEAR
    print(f"{robot} g={g}: {len(a)} edges, free {ref.mean():.3f}, mismatches {len(bad)}")


def test_device_pointers_and_edge_cases(ctx, oracle):
    import torch
    from prrtc_gb300 import PrrtcError, scenes
    from prrtc_gb300.env import Environment
    env, z = load_golden("panda_tabletop")
    q = z["q"]
    host = ctx.validate_configs("panda", env, q)
    dev = ctx.validate_configs("panda", env, torch.from_numpy(q).cuda()).cpu().numpy()
    np.testing.assert_array_equal(host, dev)
    assert len(ctx.validate_configs("panda", env, np.zeros((0, 7), np.float32))) == 0
    empty = Environment()
    free = ctx.validate_configs("panda", empty, q)
    np.testing.assert_array_equal(free, oracle.check("panda", empty, q))
    big = Environment(cuboids=np.zeros((800, 15), np.float32))
    with pytest.raises(PrrtcError):
        ctx.upload_env(big)


WEIGHTS = np.array([11, 26, 16, 27, 18, 11], np.int64)   # sphere, capsule, z-capsule, cuboid, z-cuboid, pair


@pytest.mark.parametrize("case", golden_cases())
def test_work_counts_match_oracle(case, ctx, oracle):
    """The checker's FLOP counter equals the oracle's executed-test count
    (reference hierarchy and early exits) times the roofline weights, plus the
    canonical FK count per configuration."""
    robot = case.split("_")[0]
    env, z = load_golden(case)
    q = z["q"][z["margin"] > 1e-4]          # away from contact: identical test sequences
    ctx.work_counters(reset=True)
    ctx.validate_configs(robot, env, q)
    flops, n = ctx.work_counters(reset=True)
    _, counts = oracle.check(robot, env, q, counts=True)
    from prrtc_gb300.scenes import load_model
    m = load_model(robot)
    fk = 2 * (12 * m["dof"] + 9 * len(m["spheres"]))
    assert n == len(q)
    assert flops == int(counts @ WEIGHTS) + fk * len(q)


def test_maximum_environment_and_zero_length_edges(ctx, oracle):
    """A scene of exactly PRRTC_MAX_ENV_FLOATS packed floats (all obstacle
    types) checks like the oracle, outside the near-contact bucket; an edge
    from a configuration to itself checks that configuration."""
    from prrtc_gb300 import scenes
    from prrtc_gb300.env import Environment, capsule_row, cuboid_row
    rng = np.random.default_rng(5)

    def pos(n):
        return rng.uniform([0.3, -0.8, 0.0], [1.3, 0.8, 1.4], (n, 3))

    sph = np.column_stack([pos(256), rng.uniform(0.01, 0.04, 256)]).astype(np.float32)          # 1024 floats
    caps = np.array([capsule_row(p, p + rng.uniform(-0.1, 0.1, 3), rng.uniform(0.01, 0.03)) for p in pos(128)])  # 1024
    zcaps = np.array([capsule_row(p, p + [0, 0, rng.uniform(0.05, 0.2)], rng.uniform(0.01, 0.03))
                      for p in pos(128)])                                                          # 1024
    cubs = np.array([cuboid_row(p, rng.uniform(0.01, 0.05, 3), rng.uniform(-1, 1, 3)) for p in pos(256)])       # 4096
    zcubs = np.array([cuboid_row(p, rng.uniform(0.01, 0.05, 3), (0, 0, rng.uniform(-3, 3))) for p in pos(256)])  # 4096
    env = Environment(spheres=sph, capsules=caps, z_aligned_capsules=zcaps, cuboids=cubs, z_aligned_cuboids=zcubs)
    assert env.packed_floats() == 11264
    q = scenes._uniform_configs("panda", scenes.Rng(9), 20000).astype(np.float32)
    got = ctx.validate_configs("panda", env, q)
    ref, margin = oracle.check("panda", env, q, margin=True)
    bad = np.flatnonzero(got != ref)
    assert (margin[bad] < 1e-5).all(), margin[bad]
    free = q[ref == 1][:64]
    assert len(free) > 0
    same = ctx.validate_edges("panda", env, free, free, 32)
    np.testing.assert_array_equal(same, oracle.check_edges("panda", env, free, free, 32))
    assert same.all()
