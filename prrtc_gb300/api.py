"""Python host mirror of the library's C ABI (include/prrtc/prrtc.h).

Names follow the reference: ``Settings`` has the fields of ``pRRTC_settings``
(src/planning/pRRTC_settings.hh:3-16) in the same order and with the same
defaults; ``Planner.solve`` takes (robot, start, goals, env, settings) like
``pRRTC::solve<Robot>`` (src/planning/Planners.hh:75-78) and returns a
``PlannerResult`` with the fields of the reference's ``PlannerResult<Robot>``
(Planners.hh:11-23).  Robots are named "sphere", "panda", "fetch", "baxter".

Arrays may be numpy arrays (host) or CUDA torch tensors (device memory of the
context's device, used in place).  The shared library must have been built
(``prrtc_gb300.build``); nothing here falls back to CPU code.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .env import Environment

LIB_PATH = Path(__file__).resolve().parent / "libprrtc_gb300.so"
ROBOTS = {"sphere": 0, "panda": 1, "fetch": 2, "baxter": 3}
STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "device time budget exhausted", 4: "CUDA error",
          5: "unsupported"}
_lib = None


class PrrtcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"prrtc status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class EnvDesc(C.Structure):
    _fields_ = [("spheres", C.POINTER(C.c_float)), ("num_spheres", C.c_uint32),
                ("capsules", C.POINTER(C.c_float)), ("num_capsules", C.c_uint32),
                ("z_aligned_capsules", C.POINTER(C.c_float)), ("num_z_aligned_capsules", C.c_uint32),
                ("cylinders", C.POINTER(C.c_float)), ("num_cylinders", C.c_uint32),
                ("cuboids", C.POINTER(C.c_float)), ("num_cuboids", C.c_uint32),
                ("z_aligned_cuboids", C.POINTER(C.c_float)), ("num_z_aligned_cuboids", C.c_uint32)]


class Settings(C.Structure):
    """pRRTC_settings, byte for byte."""
    _fields_ = [("max_samples", C.c_int), ("max_iters", C.c_int), ("num_new_configs", C.c_int),
                ("granularity", C.c_int), ("range", C.c_float), ("balance", C.c_int), ("tree_ratio", C.c_float),
                ("dynamic_domain", C.c_bool), ("dd_alpha", C.c_float), ("dd_radius", C.c_float),
                ("dd_min_radius", C.c_float)]

    def __init__(self, **kw):
        super().__init__()
        defaults = dict(max_samples=1000000, max_iters=1000000, num_new_configs=600, granularity=64, range=0.5,
                        balance=1, tree_ratio=0.5, dynamic_domain=True, dd_alpha=0.0001, dd_radius=4.0,
                        dd_min_radius=1.0)
        defaults.update(kw)
        for k, v in defaults.items():
            setattr(self, k, v)

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class _Result(C.Structure):
    _fields_ = [("solved", C.c_int), ("status", C.c_int), ("start_tree_size", C.c_int), ("goal_tree_size", C.c_int),
                ("path_length", C.c_int), ("iters", C.c_int), ("cost", C.c_float), ("path_rows", C.c_int),
                ("path_capacity", C.c_int), ("path", C.POINTER(C.c_float)), ("wall_ns", C.c_uint64),
                ("kernel_ns", C.c_uint64), ("copy_ns", C.c_uint64)]


@dataclass
class PlannerResult:
    """Mirror of PlannerResult<Robot> (Planners.hh:11-23); path is goal first."""
    solved: bool = False
    path: np.ndarray = field(default_factory=lambda: np.zeros((0, 0), np.float32))
    start_tree_size: int = 0
    goal_tree_size: int = 0
    path_length: int = 0
    iters: int = 0
    cost: float = 0.0
    wall_ns: int = 0
    kernel_ns: int = 0
    copy_ns: int = 0
    status: int = 0


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH.name} is not built; run `python -m prrtc_gb300.build`")
        L = C.CDLL(str(LIB_PATH))
        vp, i64, u8p, fp = C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p
        sig = {
            "prrtc_create": (C.c_int, [C.POINTER(vp), C.c_int]),
            "prrtc_destroy": (C.c_int, [vp]),
            "prrtc_status_string": (C.c_char_p, [C.c_int]),
            "prrtc_last_error": (C.c_char_p, [vp]),
            "prrtc_launch_count": (C.c_uint64, [vp]),
            "prrtc_set_planning_margin": (C.c_int, [vp, C.c_float]),
            "prrtc_set_time_budget": (C.c_int, [vp, C.c_uint64]),
            "prrtc_robot_dof": (C.c_int, [C.c_int]),
            "prrtc_robot_num_spheres": (C.c_int, [C.c_int]),
            "prrtc_robot_limits": (C.c_int, [C.c_int, fp, fp]),
            "prrtc_env_upload": (C.c_int, [vp, C.POINTER(EnvDesc), C.POINTER(vp)]),
            "prrtc_env_free": (C.c_int, [vp, vp]),
            "prrtc_validate_configs": (C.c_int, [vp, C.c_int, vp, fp, i64, u8p]),
            "prrtc_validate_edges": (C.c_int, [vp, C.c_int, vp, fp, fp, i64, C.c_int, u8p]),
            "prrtc_fk_spheres": (C.c_int, [vp, C.c_int, fp, i64, fp]),
            "prrtc_settings_default": (None, [C.POINTER(Settings)]),
            "prrtc_solve": (C.c_int, [vp, C.c_int, fp, fp, C.c_int, vp, C.POINTER(Settings), C.POINTER(_Result)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    """(pointer, keepalive) for a numpy array or a CUDA torch tensor."""
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr()), a
    a = np.ascontiguousarray(a)
    return C.c_void_p(a.ctypes.data), a


def _f32(a, cols=None):
    if hasattr(a, "data_ptr"):
        return a
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    return a.reshape(-1, cols) if cols else a


def robot_id(robot) -> int:
    return ROBOTS[robot] if isinstance(robot, str) else int(robot)


def dof(robot) -> int:
    return lib().prrtc_robot_dof(robot_id(robot))


def num_spheres(robot) -> int:
    return lib().prrtc_robot_num_spheres(robot_id(robot))


class EnvHandle:
    def __init__(self, ctx: "Context", handle: C.c_void_p, env: Environment):
        self.ctx, self.handle, self.env = ctx, handle, env

    def free(self):
        if self.handle:
            lib().prrtc_env_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.free()
        except Exception:
            pass


class Context:
    """One library context on one device (prrtc_create)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        s = lib().prrtc_create(C.byref(h), device)
        if s:
            raise PrrtcError(s, "prrtc_create failed (no CUDA device?)")
        self.handle = h

    def close(self):
        if self.handle:
            lib().prrtc_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s: int):
        if s:
            raise PrrtcError(s, lib().prrtc_last_error(self.handle).decode())

    @property
    def launches(self) -> int:
        return int(lib().prrtc_launch_count(self.handle))

    def set_planning_margin(self, pad: float):
        self._check(lib().prrtc_set_planning_margin(self.handle, pad))

    def set_time_budget(self, ns: int):
        self._check(lib().prrtc_set_time_budget(self.handle, int(ns)))

    def upload_env(self, env: Environment) -> EnvHandle:
        d = EnvDesc()
        keep = []
        for k in ("spheres", "capsules", "z_aligned_capsules", "cylinders", "cuboids", "z_aligned_cuboids"):
            a = np.ascontiguousarray(getattr(env, k), np.float32)
            keep.append(a)
            setattr(d, k, a.ctypes.data_as(C.POINTER(C.c_float)) if len(a) else None)
            setattr(d, "num_" + k, len(a))
        h = C.c_void_p()
        self._check(lib().prrtc_env_upload(self.handle, C.byref(d), C.byref(h)))
        return EnvHandle(self, h, env)

    def _env(self, env) -> EnvHandle:
        return env if isinstance(env, EnvHandle) else self.upload_env(env)

    def validate_configs(self, robot, env, q):
        """uint8 verdicts (1 = free) for configurations q [n, dof]."""
        rid = robot_id(robot)
        e = self._env(env)
        q = _f32(q, dof(rid))
        n = q.shape[0]
        out = np.empty(n, np.uint8) if not hasattr(q, "data_ptr") else _empty_like_device(q, (n,), "uint8")
        pq, kq = _ptr(q)
        po, ko = _ptr(out)
        self._check(lib().prrtc_validate_configs(self.handle, rid, e.handle, pq, n, po))
        return out

    def validate_edges(self, robot, env, a, b, granularity: int):
        rid = robot_id(robot)
        e = self._env(env)
        a, b = _f32(a, dof(rid)), _f32(b, dof(rid))
        n = a.shape[0]
        out = np.empty(n, np.uint8) if not hasattr(a, "data_ptr") else _empty_like_device(a, (n,), "uint8")
        pa, ka = _ptr(a)
        pb, kb = _ptr(b)
        po, ko = _ptr(out)
        self._check(lib().prrtc_validate_edges(self.handle, rid, e.handle, pa, pb, n, int(granularity), po))
        return out

    def fk_spheres(self, robot, q):
        """[n, num_spheres, 4] world centres and radii."""
        rid = robot_id(robot)
        q = _f32(q, dof(rid))
        n = q.shape[0]
        S = num_spheres(rid)
        out = np.empty((n, S, 4), np.float32) if not hasattr(q, "data_ptr") else _empty_like_device(q, (n, S, 4), "float32")
        pq, kq = _ptr(q)
        po, ko = _ptr(out)
        self._check(lib().prrtc_fk_spheres(self.handle, rid, pq, n, po))
        return out

    def solve(self, robot, start, goals, env, settings: Settings | None = None, path_capacity: int = 70000) -> PlannerResult:
        """pRRTC::solve<Robot>(start, goals, env, settings)."""
        rid = robot_id(robot)
        D = dof(rid)
        e = self._env(env)
        start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(D))
        goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, D))
        s = settings if settings is not None else Settings()
        path = np.empty((path_capacity, D), np.float32)
        r = _Result()
        r.path_capacity = path_capacity
        r.path = path.ctypes.data_as(C.POINTER(C.c_float))
        st = lib().prrtc_solve(self.handle, rid, start.ctypes.data_as(C.c_void_p), goals.ctypes.data_as(C.c_void_p),
                               len(goals), e.handle, C.byref(s), C.byref(r))
        if st and st != 3:
            self._check(st)
        return PlannerResult(bool(r.solved), path[:r.path_rows].copy() if r.solved else np.zeros((0, D), np.float32),
                             r.start_tree_size, r.goal_tree_size, r.path_length, r.iters, r.cost, r.wall_ns,
                             r.kernel_ns, r.copy_ns, r.status)


def _empty_like_device(t, shape, dtype: str):
    import torch
    return torch.empty(shape, dtype=getattr(torch, dtype), device=t.device)
