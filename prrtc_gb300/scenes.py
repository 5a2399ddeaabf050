"""Seeded synthetic workloads: scenes and start/goal queries.

The reference benchmarks on MotionBenchMaker problems (scripts/*.json); this
module stands in for them with seeded synthetic scenes of the same kinds and
sizes (tabletop, 3x3 shelf, mixed clutter).  No MBM item is reproduced.

Everything here is deterministic across machines: random numbers come from a
SplitMix64 stream written out below, and start/goal configurations are
accepted only when their float64 clearance (leaf spheres against obstacles and
listed self pairs, computed with numpy on the robot's fitted model) is at
least ``MIN_CLEARANCE`` — far enough from contact that every checker,
including the reference's float32 one, calls them free.  This module only
builds inputs; planning never calls it.
"""
from __future__ import annotations

import json
from dataclasses import dataclass
from functools import lru_cache
from pathlib import Path

import numpy as np

from .env import Environment, capsule_row, cuboid_row

MIN_CLEARANCE = 0.002
ROBOT_IDS = {"sphere": 0, "panda": 1, "fetch": 2, "baxter": 3}
_ROBOT_DIR = Path(__file__).resolve().parent / "robots"

# joint scaling of the reference sampler (Robots.hh get_s_m / get_s_a)
LIMITS = {
    "sphere": ([10.0, 10.0, 10.0], [-5.0, -5.0, -5.0]),
    "panda": ([5.9342, 3.6652, 5.9342, 3.2289, 5.9342, 3.9095999999999997, 5.9342],
              [-2.9671, -1.8326, -2.9671, -3.1416, -2.9671, -0.0873, -2.9671]),
    "fetch": ([0.38615, 3.2112, 2.739, 6.28318, 4.502, 6.28318, 4.32, 6.28318],
              [0.0, -1.6056, -1.221, -3.14159, -2.251, -3.14159, -2.16, -3.14159]),
    "baxter": ([3.40335987756, 3.194, 6.10835987756, 2.6679999999999997, 6.118, 3.66479632679, 6.118] * 2,
               [-1.70167993878, -2.147, -3.05417993878, -0.05, -3.059, -1.57079632679, -3.059] * 2),
}


class Rng:
    """SplitMix64 stream; uniform floats from the top 53 bits."""

    def __init__(self, seed: int):
        self.s = (int(seed) * 0x9E3779B97F4A7C15 + 0x1234567) & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0, size=None):
        if size is None:
            return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))
        n = int(np.prod(size))
        u = (self.next_u64_array(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return (np.asarray(lo) + (np.asarray(hi) - np.asarray(lo)) * u.reshape(size))

    def next_u64_array(self, n: int) -> np.ndarray:
        """The next n outputs of the stream, vectorised (uint64 arithmetic wraps)."""
        with np.errstate(over="ignore"):
            k = np.arange(1, n + 1, dtype=np.uint64)
            z = np.uint64(self.s) + k * np.uint64(0x9E3779B97F4A7C15)
            self.s = int(z[-1]) if n else self.s
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def integers(self, lo: int, hi_inclusive: int) -> int:
        return lo + int(self.next_u64() % (hi_inclusive - lo + 1))


# ------------------------------------------------------------------- scenes

def _z_one(rng: Rng, capsule: bool, lo, hi, floor_z=None):
    """One z-aligned obstacle centred uniformly in [lo, hi] (standing on the
    plane z = floor_z when given): a vertical capsule (r U[0.02, 0.05],
    length U[0.1, 0.3]) or a yawed box (half-extents U[0.02, 0.10], yaw
    U[-pi, pi]).  These are the reference's z_aligned_capsules and
    z_aligned_cuboids (environment.hh:20-30), which its checker tests with
    sphere_z_aligned_capsule / sphere_z_aligned_cuboid (utils.cuh:134-148,
    178-197): only the axis' z (capsule) or the axes' x, y (box) are read."""
    c = rng.uniform(np.asarray(lo, np.float64), np.asarray(hi, np.float64), (3,))
    if capsule:
        r = rng.uniform(0.02, 0.05)
        h = rng.uniform(0.1, 0.3)
        z0 = floor_z + r if floor_z is not None else c[2] - h / 2
        return capsule_row((c[0], c[1], z0 + h), (c[0], c[1], z0), r)
    half = rng.uniform(0.02, 0.10, (3,))
    yaw = rng.uniform(-np.pi, np.pi)
    if floor_z is not None:
        c[2] = floor_z + half[2]
    return cuboid_row(c, half, (0.0, 0.0, yaw))


def _z_extras(rng: Rng, n: int, lo, hi, floor_z=None):
    """n z-aligned obstacles, alternating capsule and box (see _z_one)."""
    rows = [_z_one(rng, k % 2 == 0, lo, hi, floor_z) for k in range(n)]
    zc = np.array([r for r in rows if len(r) == 8], np.float32).reshape(-1, 8)
    zb = np.array([r for r in rows if len(r) == 15], np.float32).reshape(-1, 15)
    return zc, zb


TABLE_CENTER = (0.8, 0.0, 0.4)
TABLE_HALF = (0.5, 0.4, 0.025)


def tabletop_scene(seed: int, z_offset: float = 0.0, n_spheres: int = 8, n_boxes: int = 4,
                   n_zaligned: int = 0) -> Environment:
    """Table (1.0 x 0.8 x 0.05 m cuboid, top at z=0.425) with spheres of radius
    U[0.03, 0.08] and axis-aligned boxes of half-extents U[0.02, 0.10] placed
    uniformly in the 0.8 m cube above it; plus n_zaligned z-aligned obstacles
    (vertical capsules and yawed boxes) standing on the table."""
    rng = Rng(seed)
    lo = np.array([0.4, -0.4, 0.425 + z_offset])
    hi = lo + 0.8
    sph = [[*rng.uniform(lo, hi, (3,)), rng.uniform(0.03, 0.08)] for _ in range(n_spheres)]
    boxes = [cuboid_row(np.array(TABLE_CENTER) + [0, 0, z_offset], TABLE_HALF)]
    for _ in range(n_boxes):
        c = rng.uniform(lo, hi, (3,))
        h = rng.uniform(0.02, 0.10, (3,))
        boxes.append(cuboid_row(c, h))
    tc = np.array(TABLE_CENTER) + [0, 0, z_offset]
    top = tc[2] + TABLE_HALF[2]
    zc, zb = _z_extras(rng, n_zaligned, tc - [0.45, 0.35, 0.0], tc + [0.45, 0.35, 0.0], floor_z=top)
    return Environment(spheres=np.array(sph, np.float32), cuboids=np.array(boxes, np.float32),
                       z_aligned_capsules=zc, z_aligned_cuboids=zb)


SHELF_FRONT_X, SHELF_DEPTH, SHELF_BOTTOM, CELL, WALL = 0.55, 0.30, 0.30, 0.25, 0.02


def shelf_cells(z_offset: float = 0.0):
    """(lo, hi) corners of the 3x3 cells' free interiors, row-major from the bottom left."""
    pitch = CELL + WALL
    width = 3 * CELL + 4 * WALL
    cells = []
    for r in range(3):
        for c in range(3):
            z0 = SHELF_BOTTOM + z_offset + WALL + r * pitch
            y0 = -width / 2 + WALL + c * pitch
            cells.append((np.array([SHELF_FRONT_X, y0, z0]), np.array([SHELF_FRONT_X + SHELF_DEPTH, y0 + CELL, z0 + CELL])))
    return cells


def shelf_scene(seed: int, z_offset: float = 0.0, n_cyl: int = 12, n_sph: int = 20, n_zaligned: int = 0) -> Environment:
    """3x3 shelf of 0.25 m cells with 0.02 m boards (4 shelves, 4 dividers and
    a back plate: 9 cuboids; front face x=0.55, depth 0.30, bottom z=0.30),
    plus vertical cylinders (r U[0.02, 0.05], h U[0.1, 0.3], random yaw;
    stored as capsules, as the reference's MBM loader stores cylinders) and
    spheres (r U[0.03, 0.08]) standing in random cells; plus n_zaligned
    z-aligned obstacles (vertical capsules, yawed boxes) standing on the
    boards of random cells."""
    rng = Rng(seed)
    pitch = CELL + WALL
    width = 3 * CELL + 4 * WALL
    height = 3 * CELL + 4 * WALL
    xc = SHELF_FRONT_X + SHELF_DEPTH / 2
    zb = SHELF_BOTTOM + z_offset
    boxes = []
    for k in range(4):     # horizontal boards
        boxes.append(cuboid_row((xc, 0.0, zb + WALL / 2 + k * pitch), (SHELF_DEPTH / 2, width / 2, WALL / 2)))
    for k in range(4):     # vertical dividers
        boxes.append(cuboid_row((xc, -width / 2 + WALL / 2 + k * pitch, zb + height / 2), (SHELF_DEPTH / 2, WALL / 2, height / 2)))
    boxes.append(cuboid_row((SHELF_FRONT_X + SHELF_DEPTH + WALL / 2, 0.0, zb + height / 2), (WALL / 2, width / 2, height / 2)))
    cells = shelf_cells(z_offset)
    caps = []
    for _ in range(n_cyl):
        lo, hi = cells[rng.integers(0, 8)]
        r = rng.uniform(0.02, 0.05)
        h = rng.uniform(0.1, 0.3)
        h = min(h, CELL - 2 * r - 1e-3)
        x = rng.uniform(lo[0] + r, hi[0] - r)
        y = rng.uniform(lo[1] + r, hi[1] - r)
        rng.uniform()  # yaw: a vertical cylinder's axis does not depend on it
        z0 = lo[2] + r
        caps.append(capsule_row((x, y, z0 + h), (x, y, z0), r))
    sph = []
    for _ in range(n_sph):
        lo, hi = cells[rng.integers(0, 8)]
        r = rng.uniform(0.03, 0.08)
        sph.append([*rng.uniform(lo + r, hi - r, (3,)), r])
    zc, zb = [], []
    for k in range(n_zaligned):
        lo, hi = cells[rng.integers(0, 8)]
        row = _z_one(rng, k % 2 == 0, lo + 0.05, hi - 0.05, floor_z=lo[2])
        (zc if len(row) == 8 else zb).append(row)
    return Environment(spheres=np.array(sph, np.float32), capsules=np.array(caps, np.float32),
                       cuboids=np.array(boxes, np.float32), z_aligned_capsules=np.array(zc, np.float32).reshape(-1, 8),
                       z_aligned_cuboids=np.array(zb, np.float32).reshape(-1, 15))


def mixed_scene(seed: int, n_obstacles: int, lo=(0.5, -0.4, 0.5), hi=(1.3, 0.4, 1.3), n_zaligned: int = 0) -> Environment:
    """n obstacles of uniformly drawn type (sphere, cuboid, capsule), sizes as
    the tabletop scene, placed uniformly in the box [lo, hi]; plus n_zaligned
    z-aligned obstacles (vertical capsules, yawed boxes) in the same box."""
    rng = Rng(seed)
    lo, hi = np.array(lo), np.array(hi)
    sph, box, cap = [], [], []
    for _ in range(n_obstacles):
        kind = rng.integers(0, 2)
        c = rng.uniform(lo, hi, (3,))
        if kind == 0:
            sph.append([*c, rng.uniform(0.03, 0.08)])
        elif kind == 1:
            box.append(cuboid_row(c, rng.uniform(0.02, 0.10, (3,)), (0.0, 0.0, rng.uniform(-np.pi, np.pi))))
        else:
            r = rng.uniform(0.02, 0.05)
            h = rng.uniform(0.1, 0.3)
            caps_dir = rng.uniform(-1.0, 1.0, (3,))
            caps_dir /= max(np.linalg.norm(caps_dir), 1e-9)
            cap.append(capsule_row(c - caps_dir * h / 2, c + caps_dir * h / 2, r))
    zc, zb = _z_extras(rng, n_zaligned, lo, hi)
    return Environment(spheres=np.array(sph, np.float32).reshape(-1, 4), cuboids=np.array(box, np.float32).reshape(-1, 15),
                       capsules=np.array(cap, np.float32).reshape(-1, 8), z_aligned_capsules=zc, z_aligned_cuboids=zb)


# ------------------------------------------------------ clearance (float64)

@lru_cache(maxsize=None)
def load_model(robot: str) -> dict:
    return json.loads((_ROBOT_DIR / f"{robot}.json").read_text())


def sphere_centres(robot: str, q: np.ndarray) -> np.ndarray:
    """(S, N, 3) float64 world centres of the model spheres."""
    from .robots.extract import model_sphere_centres
    return model_sphere_centres(load_model(robot), np.asarray(q, np.float64).reshape(-1, load_model(robot)["dof"]))


def _sd_env(env: Environment, p: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Signed distance of spheres (p (..., 3), r (...,)) to the nearest obstacle."""
    best = np.full(p.shape[:-1], np.inf)
    for s in env.spheres.astype(np.float64):
        best = np.minimum(best, np.linalg.norm(p - s[:3], axis=-1) - (r + s[3]))
    for caps, zonly in ((env.capsules, False), (env.z_aligned_capsules, True)):
        for c in caps.astype(np.float64):
            p1, v, rc, rdv = c[:3], c[3:6], c[6], c[7]
            if zonly:
                t = (p[..., 2] - p1[2]) * v[2] * rdv
            else:
                t = ((p - p1) @ v) * rdv
            t = np.clip(t, 0.0, 1.0)
            proj = p1 + t[..., None] * v if not zonly else np.stack(
                [np.full_like(t, p1[0]), np.full_like(t, p1[1]), p1[2] + v[2] * t], -1)
            best = np.minimum(best, np.linalg.norm(p - proj, axis=-1) - (r + rc))
    for cubs, zonly in ((env.cuboids, False), (env.z_aligned_cuboids, True)):
        for c in cubs.astype(np.float64):
            d = p - c[:3]
            if zonly:
                a = [np.abs(d[..., 0] * c[3] + d[..., 1] * c[4]) - c[12],
                     np.abs(d[..., 0] * c[6] + d[..., 1] * c[7]) - c[13], np.abs(d[..., 2]) - c[14]]
            else:
                a = [np.abs(d @ c[3:6]) - c[12], np.abs(d @ c[6:9]) - c[13], np.abs(d @ c[9:12]) - c[14]]
            a = [np.maximum(x, 0.0) for x in a]
            best = np.minimum(best, np.sqrt(a[0] ** 2 + a[1] ** 2 + a[2] ** 2) - r)
    return best


def clearance(robot: str, env: Environment, q: np.ndarray) -> np.ndarray:
    """Float64 clearance of each configuration: min signed distance over leaf
    spheres vs obstacles and listed leaf self pairs (< 0: penetration)."""
    return clearance_model(load_model(robot), env, q)


def clearance_model(m: dict, env: Environment, q: np.ndarray) -> np.ndarray:
    """clearance() for a model given as a dict (e.g. one built from a URDF)."""
    from .robots.extract import model_sphere_centres
    q = np.asarray(q, np.float64).reshape(-1, m["dof"])
    C = model_sphere_centres(m, q)
    R = np.array([s["r"] for s in m["spheres"]])
    leaves = sorted({l for g in m["env_groups"] for l in g["leaves"]})
    best = np.full(len(q), np.inf)
    if leaves:
        sd = _sd_env(env, C[leaves], R[leaves][:, None])
        best = np.minimum(best, sd.min(axis=0))
    pairs = np.array([p for g in m["self_groups"] for p in g["pairs"]], dtype=np.int64).reshape(-1, 2)
    if len(pairs):
        d = np.linalg.norm(C[pairs[:, 0]] - C[pairs[:, 1]], axis=-1) - (R[pairs[:, 0]] + R[pairs[:, 1]])[:, None]
        best = np.minimum(best, d.min(axis=0))
    return best


# ------------------------------------------------------------------ queries

@dataclass
class Query:
    env: Environment
    start: np.ndarray
    goal: np.ndarray
    seed: int
    kind: str


def _uniform_configs(robot: str, rng: Rng, n: int) -> np.ndarray:
    scale, offset = (np.array(v, np.float64) for v in LIMITS[robot])
    u = rng.uniform(0.0, 1.0, (n, len(scale)))
    return (u * scale + offset).astype(np.float32)


def sample_free(robot: str, env: Environment, rng: Rng, accept=None, batch: int = 64, max_batches: int = 2000) -> np.ndarray:
    """First configuration (in stream order) with clearance >= MIN_CLEARANCE
    that also passes accept(q_batch) -> bool mask."""
    for _ in range(max_batches):
        q = _uniform_configs(robot, rng, batch)
        ok = np.ones(batch, bool)
        if accept is not None:
            ok &= accept(q)
        idx = np.flatnonzero(ok)
        if len(idx):
            cl = clearance(robot, env, q[idx])
            good = idx[cl >= MIN_CLEARANCE]
            if len(good):
                return q[good[0]]
    raise RuntimeError("no free configuration found")


def hand_sphere(robot: str) -> int:
    """Index of the end-effector bounding sphere (the last gated env group)."""
    m = load_model(robot)
    gated = [g for g in m["env_groups"] if g["gate"] >= 0]
    return gated[-1]["gate"]


def in_cell(robot: str, q: np.ndarray, cell) -> np.ndarray:
    from .robots.extract import model_sphere_centres
    lo, hi = cell
    c = model_sphere_centres(load_model(robot), np.asarray(q, np.float64), only=[hand_sphere(robot)])[0]
    return np.all((c >= lo) & (c <= hi), axis=-1)


def make_query(robot: str, kind: str, seed: int, n_obstacles: int | None = None, z_offset: float = 0.0,
               n_zaligned: int = 0) -> Query:
    """One seeded query.  kind: 'tabletop', 'shelf' (goal: hand inside a cell)
    or 'mixed' (n_obstacles of mixed types); n_zaligned adds that many
    z-aligned obstacles to the scene."""
    if kind == "tabletop":
        env = tabletop_scene(seed, z_offset, n_zaligned=n_zaligned)
    elif kind == "shelf":
        env = shelf_scene(seed, z_offset, n_zaligned=n_zaligned)
    elif kind == "mixed":
        env = mixed_scene(seed, n_obstacles if n_obstacles is not None else 20, n_zaligned=n_zaligned)
    else:
        raise ValueError(kind)
    rng = Rng(seed ^ 0x5A5A5A5A)
    start = sample_free(robot, env, rng)
    if kind == "shelf":
        # goal: hand inside a random cell; a cell the hand cannot reach free of
        # collision within the attempt budget gives way to the next draw
        cells = shelf_cells(z_offset)
        goal = None
        for _ in range(16):
            cell = cells[rng.integers(0, 8)]
            try:
                goal = sample_free(robot, env, rng, accept=lambda q: in_cell(robot, q, cell), batch=4096,
                                   max_batches=60)
                break
            except RuntimeError:
                continue
        if goal is None:
            raise RuntimeError(f"no reachable shelf cell for {robot} seed {seed}")
    else:
        goal = sample_free(robot, env, rng)
    return Query(env, start, goal, seed, kind)
