"""ctypes binding of the oracle (test infrastructure only; see oracle.h).

``OracleLib`` wraps oracle/liboracle.so (the C restatement); ``RefLib``
wraps oracle/_ref/libref_fkcc.so (pRRTC's own checker compiled from its
sources by `make -C oracle ref`, present only where the reference is).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROBOTS = {"sphere": 0, "panda": 1, "fetch": 2, "baxter": 3}
REF_NAMES = {"sphere": "Sphere", "panda": "Panda", "fetch": "Fetch", "baxter": "Baxter"}


class OEnv(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("ns", C.c_int), ("capsules", C.c_void_p), ("nc", C.c_int),
                ("zcapsules", C.c_void_p), ("nzc", C.c_int), ("cuboids", C.c_void_p), ("ncb", C.c_int),
                ("zcuboids", C.c_void_p), ("nzb", C.c_int)]


class OSettings(C.Structure):
    _fields_ = [("max_samples", C.c_int), ("max_iters", C.c_int), ("num_new_configs", C.c_int),
                ("granularity", C.c_int), ("range", C.c_float), ("balance", C.c_int), ("tree_ratio", C.c_float),
                ("dynamic_domain", C.c_int), ("dd_alpha", C.c_float), ("dd_radius", C.c_float),
                ("dd_min_radius", C.c_float), ("budget_s", C.c_double)]


class OResult(C.Structure):
    _fields_ = [("solved", C.c_int), ("start_tree_size", C.c_int), ("goal_tree_size", C.c_int),
                ("path_length", C.c_int), ("path_rows", C.c_int), ("iters", C.c_int), ("cost", C.c_float),
                ("checks", C.c_int64)]


def _arr(a, cols):
    a = np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, cols))
    return a


class _EnvRef:
    """Keeps the arrays of an oracle_env alive."""

    def __init__(self, env):
        self.arrs = [_arr(env.spheres, 4), _arr(env.capsules, 8), _arr(env.z_aligned_capsules, 8),
                     _arr(env.cuboids, 15), _arr(env.z_aligned_cuboids, 15)]
        s, c, zc, cb, zcb = self.arrs
        self.s = OEnv(s.ctypes.data, len(s), c.ctypes.data, len(c), zc.ctypes.data, len(zc), cb.ctypes.data, len(cb),
                      zcb.ctypes.data, len(zcb))


def build(ref: bool = False):
    subprocess.run(["make", "-s", "-C", str(HERE)] + (["ref"] if ref else []), check=True)


class OracleLib:
    def __init__(self):
        p = HERE / "liboracle.so"
        if not p.exists():
            build()
        self.L = C.CDLL(str(p))
        self.L.oracle_check.argtypes = [C.c_int, C.c_void_p, C.c_long, C.POINTER(OEnv), C.c_void_p, C.c_void_p, C.c_void_p]
        self.L.oracle_check_edges.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.POINTER(OEnv), C.c_void_p]
        self.L.oracle_clearance.argtypes = [C.c_int, C.c_void_p, C.c_long, C.POINTER(OEnv), C.c_void_p]
        self.L.oracle_cost_grad.argtypes = [C.c_int, C.c_void_p, C.c_long, C.POINTER(OEnv), C.c_double, C.c_void_p,
                                            C.c_void_p]
        self.L.oracle_fk_spheres.argtypes = [C.c_int, C.c_void_p, C.c_long, C.c_void_p]
        self.L.oracle_solve.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(OEnv), C.POINTER(OSettings),
                                        C.c_void_p, C.c_void_p, C.c_int, C.POINTER(OResult)]
        self.L.oracle_solve_many.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(OSettings),
                                             C.c_void_p, C.c_int, C.c_void_p, C.c_int]

    def dof(self, robot):
        return self.L.oracle_dof(ROBOTS[robot])

    def check(self, robot, env, q, margin=False, counts=False):
        D = self.dof(robot)
        q = _arr(q, D)
        e = _EnvRef(env)
        out = np.empty(len(q), np.uint8)
        m = np.empty(len(q), np.float64) if margin else None
        c = np.zeros(6, np.int64) if counts else None
        rc = self.L.oracle_check(ROBOTS[robot], q.ctypes.data, len(q), C.byref(e.s), out.ctypes.data,
                                 m.ctypes.data if margin else None, c.ctypes.data if counts else None)
        assert rc == 0
        res = [out]
        if margin:
            res.append(m)
        if counts:
            res.append(c)
        return res[0] if len(res) == 1 else tuple(res)

    def check_edges(self, robot, env, a, b, g):
        D = self.dof(robot)
        a, b = _arr(a, D), _arr(b, D)
        e = _EnvRef(env)
        out = np.empty(len(a), np.uint8)
        assert self.L.oracle_check_edges(ROBOTS[robot], a.ctypes.data, b.ctypes.data, len(a), g, C.byref(e.s), out.ctypes.data) == 0
        return out

    def clearance(self, robot, env, q):
        D = self.dof(robot)
        q = _arr(q, D)
        e = _EnvRef(env)
        out = np.empty(len(q), np.float64)
        assert self.L.oracle_clearance(ROBOTS[robot], q.ctypes.data, len(q), C.byref(e.s), out.ctypes.data) == 0
        return out

    def cost_grad(self, robot, env, q, margin):
        """Float64 clearance cost [n] and gradient [n][dof] of configurations q (float64)."""
        D = self.dof(robot)
        q = np.ascontiguousarray(np.asarray(q, np.float64).reshape(-1, D))
        e = _EnvRef(env)
        cost = np.empty(len(q), np.float64)
        grad = np.empty((len(q), D), np.float64)
        assert self.L.oracle_cost_grad(ROBOTS[robot], q.ctypes.data, len(q), C.byref(e.s), float(margin),
                                       cost.ctypes.data, grad.ctypes.data) == 0
        return cost, grad

    def fk_spheres(self, robot, q):
        D = self.dof(robot)
        q = np.ascontiguousarray(np.asarray(q, np.float64).reshape(-1, D))
        S = self.L.oracle_num_spheres(ROBOTS[robot])
        out = np.empty((len(q), S, 4), np.float64)
        assert self.L.oracle_fk_spheres(ROBOTS[robot], q.ctypes.data, len(q), out.ctypes.data) == 0
        return out

    @staticmethod
    def settings(s, budget_s: float = 0.0) -> OSettings:
        d = dict(s if isinstance(s, dict) else s.as_dict())
        d.setdefault("budget_s", budget_s)
        o = OSettings()
        for k, _ in OSettings._fields_:
            setattr(o, k, int(d[k]) if k == "dynamic_domain" else d[k])
        return o

    def solve(self, robot, start, goals, env, settings, bases=None, path_cap=70000):
        D = self.dof(robot)
        start = _arr(start, D)
        goals = _arr(goals, D)
        e = _EnvRef(env)
        path = np.empty((path_cap, D), np.float32)
        r = OResult()
        b = None if bases is None else np.ascontiguousarray(np.asarray(bases, np.float32))
        rc = self.L.oracle_solve(ROBOTS[robot], start.ctypes.data, goals.ctypes.data, len(goals), C.byref(e.s),
                                 C.byref(self.settings(settings)), b.ctypes.data if b is not None else None,
                                 path.ctypes.data, path_cap, C.byref(r))
        assert rc == 0
        return r, path[:r.path_rows].copy() if r.solved else None

    def solve_many(self, robot, starts, goals, envs, settings, threads=0, path_cap=4096, budget_s=0.0):
        D = self.dof(robot)
        starts, goals = _arr(starts, D), _arr(goals, D)
        refs = [_EnvRef(e) for e in envs]
        earr = (OEnv * len(refs))(*[r.s for r in refs])
        res = (OResult * len(refs))()
        paths = np.empty((len(refs), path_cap, D), np.float32)
        rc = self.L.oracle_solve_many(ROBOTS[robot], len(refs), starts.ctypes.data, goals.ctypes.data, earr,
                                      C.byref(self.settings(settings, budget_s)), paths.ctypes.data, path_cap, res, threads)
        assert rc == 0
        return list(res), paths


class RefLib:
    """pRRTC's own fkcc<Robot>, host-compiled from the reference sources."""

    PATH = HERE / "_ref" / "libref_fkcc.so"

    def __init__(self):
        self.L = C.CDLL(str(self.PATH))
        for r in REF_NAMES.values():
            f = getattr(self.L, f"ref_fkcc_{r}")
            f.argtypes = [C.c_void_p, C.c_long, C.c_int] + [C.c_void_p, C.c_int] * 5 + [C.c_void_p]
            f.restype = C.c_int

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()

    def check(self, robot, env, q):
        D = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]
        q = _arr(q, D)
        e = _EnvRef(env)
        s, c, zc, cb, zcb = e.arrs
        out = np.empty(len(q), np.uint8)
        rc = getattr(self.L, f"ref_fkcc_{REF_NAMES[robot]}")(q.ctypes.data, len(q), D, s.ctypes.data, len(s),
                                                             c.ctypes.data, len(c), zc.ctypes.data, len(zc),
                                                             cb.ctypes.data, len(cb), zcb.ctypes.data, len(zcb),
                                                             out.ctypes.data)
        assert rc == 0
        return out
