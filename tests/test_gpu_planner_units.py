"""Unit parity of the planner's device pieces against the oracle (and, where
pRRTC's own sampler was compiled from the reference sources, against it).

* Halton sampling (pRRTC.cu:81-105, Robots.hh scale_cfg): 600 lanes x 10^4
  points per robot, bit-exact, raw and scaled, from the library's cuRAND
  bases (shuffle_array, pRRTC.cu:49-56).
* Nearest neighbour (pRRTC.cu:384-412,478-505): indices and squared
  distances bit-exact for the warp and block scans, including exact ties
  (lowest index wins), NaN (in-flight) nodes and ragged counts.
* Dynamic domain (pRRTC.cu:456-468,584-598): radii bit-exact after seeded
  grow/shrink sequences, and after 1024 contending updates of one radius.

The harness (tests/cuda/planner_units.cu) runs the library's own device
functions; it is compiled here with nvcc against the library.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
FLT_MAX = np.float32(3.4028234663852886e38)


@pytest.fixture(scope="module")
def units(ctx):
    import prrtc_gb300.build as b
    src = ROOT / "tests" / "cuda" / "planner_units.cu"
    out_dir = ROOT / "tests" / "cuda" / "_build"
    out_dir.mkdir(exist_ok=True)
    so = out_dir / "libplanner_units.so"
    if not so.exists() or so.stat().st_mtime < max(src.stat().st_mtime, b.LIB.stat().st_mtime):
        cmd = [b.NVCC, *b.ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared",
               f"-I{b.CSRC}", f"-I{ROOT / 'include'}", str(src), "-o", str(so), f"-L{b.PKG}", "-lprrtc_gb300",
               f"-Xlinker", f"-rpath,{b.PKG}"]
        subprocess.run(cmd, check=True)
    L = C.CDLL(str(so))
    for f in ("units_halton_bases", "units_halton", "units_nearest", "units_dd_seq", "units_dd_contend"):
        getattr(L, f).restype = C.c_int
    L.units_dd_seq.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float]
    L.units_dd_contend.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]
    return L


def _p(t):
    return C.c_void_p(t.data_ptr())


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


ROBOT_DOF = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}


@pytest.mark.parametrize("robot", ["panda", "fetch", "baxter", "sphere"])
def test_halton_sequence_matches_oracle_and_reference(robot, units, oracle):
    import torch
    from prrtc_gb300 import scenes
    lanes, steps, D = 600, 10_000, ROBOT_DOF[robot]
    bases = torch.empty((lanes, 16), dtype=torch.float32, device="cuda")
    assert units.units_halton_bases(_p(bases), lanes) == 0
    scale = torch.tensor(scenes.LIMITS[robot][0], dtype=torch.float32, device="cuda")
    offset = torch.tensor(scenes.LIMITS[robot][1], dtype=torch.float32, device="cuda")
    raw = torch.empty((lanes, steps, D), dtype=torch.float32, device="cuda")
    cfg = torch.empty_like(raw)
    assert units.units_halton(D, _p(bases), lanes, steps, _p(scale), _p(offset), _p(raw), _p(cfg)) == 0
    b = bases.cpu().numpy()
    # every lane's bases are a permutation of the 16 primes; lane 0 is unshuffled
    primes = np.array([3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59], np.float32)
    assert (np.sort(b, 1) == primes).all() and (b[0] == primes).all()
    o_raw, o_cfg = oracle.halton(b, steps, scale.cpu().numpy(), offset.cpu().numpy())
    np.testing.assert_array_equal(_bits(raw.cpu().numpy()), _bits(o_raw))
    np.testing.assert_array_equal(_bits(cfg.cpu().numpy()), _bits(o_cfg))
    from pyoracle import RefSampler
    if not RefSampler.available():
        print(f"{robot}: {lanes} lanes x {steps} points bit-exact with the oracle (pRRTC's sampler not built)")
        return
    r_bases, r_raw, r_cfg = RefSampler().run(robot, lanes, steps)
    np.testing.assert_array_equal(b[:, :D], r_bases)
    np.testing.assert_array_equal(_bits(raw.cpu().numpy()), _bits(r_raw))
    np.testing.assert_array_equal(_bits(cfg.cpu().numpy()), _bits(r_cfg))
    print(f"{robot}: {lanes} lanes x {steps} points bit-exact with the oracle and with pRRTC's own sampler")


def _tree(rng, D, count, cap, dup=0, nan=0):
    """SoA tree [D][cap]: count nodes, `dup` of them copies of earlier nodes
    (exact ties), `nan` of them partly unwritten (NaN in one coordinate, as an
    in-flight append), everything past count NaN (the arena's fill)."""
    rows = rng.uniform(-3, 3, (count, D)).astype(np.float32)
    if count > 1 and dup:
        src = rng.integers(0, count - 1, dup)
        dst = np.array([rng.integers(s + 1, count) for s in src])
        rows[dst] = rows[src]
    if nan:
        idx = rng.integers(0, count, nan)
        rows[idx, rng.integers(0, D, nan)] = np.nan
    soa = np.full((D, cap), np.nan, np.float32)
    soa[:, :count] = rows.T
    return rows, soa


@pytest.mark.parametrize("D", [3, 7, 8, 14])
@pytest.mark.parametrize("count", [1, 2, 5, 31, 32, 33, 1000, 40_001])
def test_nearest_matches_oracle(D, count, units, oracle):
    import torch
    rng = np.random.default_rng(D * 100_003 + count)
    cap = (count + 3) // 4 * 4 + 4 * int(rng.integers(0, 3))
    rows, soa = _tree(rng, D, count, cap, dup=min(count // 3, 200), nan=min(count // 10, 50))
    nq = 512
    q = rng.uniform(-3, 3, (nq, D)).astype(np.float32)
    finite = np.flatnonzero(np.isfinite(rows).all(1))
    if len(finite):
        q[: nq // 4] = rows[rng.choice(finite, nq // 4)]     # distance 0, often tied with a duplicate
    want_i, want_d = oracle.nearest(rows, q)
    t_nodes = torch.from_numpy(soa).cuda()
    t_q = torch.from_numpy(q).cuda()
    out = [torch.empty(nq, dtype=dt, device="cuda") for dt in (torch.int32, torch.float32) * 2]
    for block in (32, 128, 256):
        assert units.units_nearest(D, _p(t_nodes), cap, count, _p(t_q), nq, block, *[_p(o) for o in out]) == 0
        wi, wd, bi, bd = (o.cpu().numpy() for o in out)
        np.testing.assert_array_equal(wi, want_i)
        np.testing.assert_array_equal(_bits(wd), _bits(want_d))
        np.testing.assert_array_equal(bi, want_i)
        np.testing.assert_array_equal(_bits(bd), _bits(want_d))


@pytest.mark.parametrize("alpha,r0,rmin", [(1e-4, 4.0, 1.0), (0.1, 2.0, 0.5), (0.5, 1.0, 0.01)])
def test_dynamic_domain_matches_oracle(alpha, r0, rmin, units, oracle):
    import torch
    rng = np.random.default_rng(int(alpha * 1e6))
    n, k = 4096, 64
    radii = rng.uniform(0.2, 6.0, n).astype(np.float32)
    radii[rng.random(n) < 0.25] = FLT_MAX                 # nodes whose domain is still unbounded
    ops = (rng.random((n, k)) < rng.random((n, 1))).astype(np.uint8)   # per-radius shrink probability
    want = oracle.dd_apply(radii, ops, alpha, r0, rmin)
    t_r = torch.from_numpy(radii.copy()).cuda()
    t_ops = torch.from_numpy(ops).cuda()
    assert units.units_dd_seq(_p(t_r), n, _p(t_ops), k, alpha, r0, rmin) == 0
    np.testing.assert_array_equal(_bits(t_r.cpu().numpy()), _bits(want))
    # 1024 concurrent updates of one radius: every one lands (same ops in any order give one result)
    for op, start in ((0, np.float32(1.0)), (1, FLT_MAX), (1, np.float32(5.0))):
        t1 = torch.tensor([start], dtype=torch.float32, device="cuda")
        assert units.units_dd_contend(_p(t1), 1024, op, alpha, r0, rmin) == 0
        seq = oracle.dd_apply(np.array([start], np.float32), np.full((1, 1024), op, np.uint8), alpha, r0, rmin)
        np.testing.assert_array_equal(_bits(t1.cpu().numpy()), _bits(seq))
