"""Obstacle environments in the reference's data model.

Mirrors ``ppln::collision::Environment<float>`` (src/collision/environment.hh:11-44)
as flat float32 arrays, one row per obstacle, in the layouts of the C ABI
(include/prrtc/prrtc.h):

=====================  ====  ===========================================
field                  cols  row
=====================  ====  ===========================================
``spheres``            4     x y z r
``capsules``           8     x1 y1 z1 xv yv zv r rdv
``z_aligned_capsules`` 8     same, axis along z
``cylinders``          8     same; kept but never checked, as in pRRTC
``cuboids``            15    x y z, axis_1 xyz, axis_2 xyz, axis_3 xyz, r1 r2 r3
``z_aligned_cuboids``  15    same
=====================  ====  ===========================================
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_COLS = {"spheres": 4, "capsules": 8, "z_aligned_capsules": 8, "cylinders": 8, "cuboids": 15,
         "z_aligned_cuboids": 15}


def _empty(k):
    return np.zeros((0, _COLS[k]), np.float32)


@dataclass
class Environment:
    spheres: np.ndarray = field(default_factory=lambda: _empty("spheres"))
    capsules: np.ndarray = field(default_factory=lambda: _empty("capsules"))
    z_aligned_capsules: np.ndarray = field(default_factory=lambda: _empty("z_aligned_capsules"))
    cylinders: np.ndarray = field(default_factory=lambda: _empty("cylinders"))
    cuboids: np.ndarray = field(default_factory=lambda: _empty("cuboids"))
    z_aligned_cuboids: np.ndarray = field(default_factory=lambda: _empty("z_aligned_cuboids"))

    def __post_init__(self):
        for k, c in _COLS.items():
            a = np.ascontiguousarray(np.asarray(getattr(self, k), np.float32).reshape(-1, c))
            setattr(self, k, a)

    @property
    def num_obstacles(self) -> int:
        return sum(len(getattr(self, k)) for k in _COLS if k != "cylinders")

    def packed_floats(self) -> int:
        return 4 * len(self.spheres) + 8 * (len(self.capsules) + len(self.z_aligned_capsules)) + \
            16 * (len(self.cuboids) + len(self.z_aligned_cuboids))

    def digest(self) -> str:
        import hashlib
        h = hashlib.sha256()
        for k in _COLS:
            h.update(k.encode())
            h.update(getattr(self, k).tobytes())
        return h.hexdigest()[:16]


def capsule_row(p1, p2, r):
    """Capsule between endpoints p1 and p2, computed as the reference's factory
    does (factory.hh:238-249): v = p2 - p1 and |v|^2 in float32, then
    rdv = 1 / |v|^2 in float64 rounded to float32."""
    p1 = np.asarray(p1, np.float32)
    v = np.asarray(p2, np.float32) - p1
    dot = np.float32(v[0] * v[0]) + np.float32(v[1] * v[1])
    dot = np.float32(dot + np.float32(v[2] * v[2]))
    rdv = np.float32(1.0 / float(dot))
    return np.array([*p1, *v, r, rdv], np.float32)


def euler_xyz_matrix(roll, pitch, yaw):
    """Rotation R = Rz(yaw) Ry(pitch) Rx(roll), the reference factory's
    convention for Euler XYZ (factory.hh:39-45)."""
    cr, sr = np.cos(roll), np.sin(roll)
    cp, sp = np.cos(pitch), np.sin(pitch)
    cy, sy = np.cos(yaw), np.sin(yaw)
    rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    return rz @ ry @ rx


def cuboid_row(center, half_extents, rpy=(0.0, 0.0, 0.0)):
    """Oriented box: axes are the columns of the Euler-XYZ rotation
    (factory.hh:28-63)."""
    R = euler_xyz_matrix(*rpy)
    return np.array([*center, *R[:, 0], *R[:, 1], *R[:, 2], *half_extents], np.float32)


def cylinder_capsule_row(center, rpy, length, radius):
    """Cylinder given by centre, Euler XYZ and length, as the reference's
    factory turns it into endpoints: p1 = centre + R (0, 0, L/2), p2 = centre
    - R (0, 0, L/2) (factory.hh cylinder::center::flat); the MBM loader
    stores the result in the capsules array (evaluate_mbm.cpp:40-53)."""
    R = euler_xyz_matrix(*rpy)
    axis = R[:, 2] * (length / 2.0)
    c = np.asarray(center, np.float64)
    return capsule_row(c + axis, c - axis, radius)
