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
    # const float * fields held as addresses (same size and layout as the C struct)
    _fields_ = [("spheres", C.c_void_p), ("num_spheres", C.c_uint32),
                ("capsules", C.c_void_p), ("num_capsules", C.c_uint32),
                ("z_aligned_capsules", C.c_void_p), ("num_z_aligned_capsules", C.c_uint32),
                ("cylinders", C.c_void_p), ("num_cylinders", C.c_uint32),
                ("cuboids", C.c_void_p), ("num_cuboids", C.c_uint32),
                ("z_aligned_cuboids", C.c_void_p), ("num_z_aligned_cuboids", C.c_uint32)]


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
                ("kernel_ns", C.c_uint64), ("copy_ns", C.c_uint64), ("finish_ns", C.c_uint64),
                ("samples", C.c_int64)]


class _Query(C.Structure):
    _fields_ = [("env", C.c_void_p), ("env_desc", C.c_void_p), ("start", C.c_void_p), ("goals", C.c_void_p),
                ("num_goals", C.c_int)]


class BatchSettings(C.Structure):
    """prrtc_batch_settings: planner settings for every query plus the batch's
    arena, launch shape, CUDA-graph and margin options."""
    _fields_ = [("plan", Settings), ("lanes", C.c_int), ("max_nodes_per_tree", C.c_int), ("max_active", C.c_int),
                ("warps_per_block", C.c_int), ("edge_order", C.c_int), ("sampler", C.c_int),
                ("max_attempts", C.c_int), ("restart_after_ns", C.c_uint64), ("max_workers_per_attempt", C.c_int),
                ("blocks_per_sm", C.c_int),
                ("use_graph", C.c_int),
                ("margin", C.c_float), ("time_budget_ns", C.c_uint64), ("admission", C.c_int),
                ("idle_wait_limit", C.c_uint32), ("shared_frames", C.c_int),
                ("rounds_per_header", C.c_int)]

    def __init__(self, plan: Settings | None = None, **kw):
        super().__init__()
        self.plan = plan if plan is not None else Settings()
        self.time_budget_ns = int(60e9)     # a guard for interactive use; 0 = unbounded (the C default)
        for k, v in kw.items():
            setattr(self, k, v)


class SmoothSettings(C.Structure):
    """prrtc_smooth_settings."""
    _fields_ = [("margin", C.c_float), ("steps", C.c_int), ("step", C.c_float), ("cost_weight", C.c_float),
                ("smooth_weight", C.c_float), ("granularity", C.c_int), ("shortcut_rounds", C.c_int)]

    def __init__(self, **kw):
        super().__init__()
        lib().prrtc_smooth_settings_default(C.byref(self))
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)


class _BatchStats(C.Structure):
    _fields_ = [("kernel_ns", C.c_uint64), ("samples", C.c_int64), ("solved", C.c_int), ("blocks", C.c_int),
                ("warps_per_block", C.c_int), ("slots", C.c_int), ("error", C.c_int), ("extra_attempts", C.c_int),
                ("configs_checked", C.c_uint64), ("flops", C.c_uint64), ("nn_nodes", C.c_uint64),
                ("bulk_ns", C.c_uint64), ("bulk_flops", C.c_uint64), ("bulk_configs", C.c_uint64)]


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
    finish_ns: int = 0       # batched form: launch start to this query's end (device clock)
    samples: int = 0         # batched form: samples drawn, all attempts


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
            "prrtc_sample_goals": (C.c_int, [vp, C.c_int, vp, C.c_int, fp, fp, C.c_uint64, i64, C.c_int, fp,
                                             C.POINTER(C.c_int)]),
            "prrtc_settings_default": (None, [C.POINTER(Settings)]),
            "prrtc_solve": (C.c_int, [vp, C.c_int, fp, fp, C.c_int, vp, C.POINTER(Settings), C.POINTER(_Result)]),
            "prrtc_measure_fp32_peak": (C.c_int, [vp, C.POINTER(C.c_double)]),
            "prrtc_work_counters": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int]),
            "prrtc_last_kernel_ns": (C.c_int, [vp, C.POINTER(C.c_uint64)]),
            "prrtc_batch_settings_default": (None, [C.POINTER(BatchSettings)]),
            "prrtc_batch_create": (C.c_int, [vp, C.c_int, C.POINTER(_Query), C.c_int, C.POINTER(BatchSettings), C.POINTER(vp)]),
            "prrtc_batch_run": (C.c_int, [vp, vp]),
            "prrtc_batch_results": (C.c_int, [vp, vp, C.POINTER(_Result)]),
            "prrtc_batch_stats_get": (C.c_int, [vp, vp, C.POINTER(_BatchStats)]),
            "prrtc_batch_free": (C.c_int, [vp, vp]),
            "prrtc_solve_batch": (C.c_int, [vp, C.c_int, C.POINTER(_Query), C.c_int, C.POINTER(BatchSettings), C.POINTER(_Result)]),
            "prrtc_path_cost_grad": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.c_int, C.c_int, fp, C.c_float, fp, fp]),
            "prrtc_smooth_settings_default": (None, [C.POINTER(SmoothSettings)]),
            "prrtc_smooth_paths": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.c_int, C.c_int, fp, C.POINTER(SmoothSettings),
                                             u8p, fp, fp]),
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

    def measure_fp32_peak(self) -> float:
        """FP32 FMA throughput of the device, TFLOP/s."""
        v = C.c_double()
        self._check(lib().prrtc_measure_fp32_peak(self.handle, C.byref(v)))
        return v.value

    def work_counters(self, reset: bool = False) -> tuple:
        """(algorithmic FLOPs, configurations) checked since the last reset."""
        f, n = C.c_uint64(), C.c_uint64()
        self._check(lib().prrtc_work_counters(self.handle, C.byref(f), C.byref(n), int(reset)))
        return f.value, n.value

    def last_kernel_ns(self) -> int:
        """Device time of the last validate_configs / validate_edges kernel."""
        v = C.c_uint64()
        self._check(lib().prrtc_last_kernel_ns(self.handle, C.byref(v)))
        return v.value

    def set_planning_margin(self, pad: float):
        self._check(lib().prrtc_set_planning_margin(self.handle, pad))

    def set_time_budget(self, ns: int):
        self._check(lib().prrtc_set_time_budget(self.handle, int(ns)))

    def upload_env(self, env: Environment) -> EnvHandle:
        d, keep = _env_desc(env)
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

    def sample_goals(self, robot, env, sphere: int, box_lo, box_hi, max_goals: int = 8, tries: int = 1 << 20,
                     seed: int = 0) -> np.ndarray:
        """[k, dof] collision-free configurations (k <= max_goals) whose model
        sphere `sphere` has its centre inside the box (prrtc_sample_goals)."""
        rid = robot_id(robot)
        e = self._env(env)
        lo = np.ascontiguousarray(np.asarray(box_lo, np.float32).reshape(3))
        hi = np.ascontiguousarray(np.asarray(box_hi, np.float32).reshape(3))
        out = np.empty((max(max_goals, 1), dof(rid)), np.float32)
        k = C.c_int()
        self._check(lib().prrtc_sample_goals(self.handle, rid, e.handle, int(sphere), C.c_void_p(lo.ctypes.data),
                                             C.c_void_p(hi.ctypes.data), int(seed), int(tries), int(max_goals),
                                             C.c_void_p(out.ctypes.data), C.byref(k)))
        return out[:k.value].copy()

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

    def _env_table(self, envs, n_paths: int):
        seen = {}   # one upload per distinct environment object
        hs = []
        for e in (envs if isinstance(envs, (list, tuple)) else [envs] * n_paths):
            if id(e) not in seen:
                seen[id(e)] = self._env(e)
            hs.append(seen[id(e)])
        if len(hs) != n_paths:
            raise ValueError(f"{len(hs)} environments for {n_paths} paths")
        return (C.c_void_p * n_paths)(*[h.handle.value for h in hs]), hs

    def path_cost_grad(self, robot, envs, q, margin: float = 0.02):
        """Clearance cost [P, W] and gradient [P, W, dof] of paths q [P, W, dof]
        (numpy or CUDA tensor); envs: one environment per path, or one for all."""
        rid = robot_id(robot)
        D = dof(rid)
        dev = hasattr(q, "data_ptr")
        q = q.contiguous() if dev else np.ascontiguousarray(np.asarray(q, np.float32))
        P, W = q.shape[0], q.shape[1]
        assert q.shape[2] == D
        table, keep = self._env_table(envs, P)
        if dev:
            cost, grad = _empty_like_device(q, (P, W), "float32"), _empty_like_device(q, (P, W, D), "float32")
        else:
            cost, grad = np.empty((P, W), np.float32), np.empty((P, W, D), np.float32)
        pq, kq = _ptr(q)
        pc, kc = _ptr(cost)
        pg, kg = _ptr(grad)
        self._check(lib().prrtc_path_cost_grad(self.handle, rid, table, P, W, pq, float(margin), pc, pg))
        return cost, grad

    def smooth_paths(self, robot, envs, q, settings: SmoothSettings | None = None):
        """Smooths paths q [P, W, dof] (numpy: a smoothed copy is returned; CUDA
        tensor: smoothed in place).  Returns (q, accepted[P], cost_before[P],
        cost_after[P]); rejected paths are returned unchanged."""
        rid = robot_id(robot)
        D = dof(rid)
        s = settings if settings is not None else SmoothSettings()
        dev = hasattr(q, "data_ptr")
        q = q.contiguous() if dev else np.array(q, np.float32, copy=True, order="C")
        P, W = q.shape[0], q.shape[1]
        assert q.shape[2] == D
        table, keep = self._env_table(envs, P)
        if dev:
            acc = _empty_like_device(q, (P,), "uint8")
            cb, ca = _empty_like_device(q, (P,), "float32"), _empty_like_device(q, (P,), "float32")
        else:
            acc, cb, ca = np.empty(P, np.uint8), np.empty(P, np.float32), np.empty(P, np.float32)
        pq, kq = _ptr(q)
        pa, ka = _ptr(acc)
        pb, kb = _ptr(cb)
        pc, kc = _ptr(ca)
        self._check(lib().prrtc_smooth_paths(self.handle, rid, table, P, W, pq, C.byref(s), pa, pb, pc))
        return q, acc, cb, ca

    def batch(self, robot, queries, settings: BatchSettings | None = None, path_capacity: int = 4096) -> Batch:
        """Prepare a batch; queries are (env, start, goals) tuples or objects
        with env/start/goal attributes (env: Environment or EnvHandle)."""
        return Batch(self, robot, queries, settings if settings is not None else BatchSettings(), path_capacity)

    def solve_batch(self, robot, queries, settings: BatchSettings | None = None, path_capacity: int = 4096) -> list:
        """prrtc_solve_batch: upload, solve and download in one call."""
        prep = self.prepare_batch(robot, queries, path_capacity)
        self.solve_prepared(prep, settings)
        return prep.results()

    def prepare_batch(self, robot, queries, path_capacity: int = 4096) -> "PreparedBatch":
        """The host side of prrtc_solve_batch's arguments: the prrtc_query
        array (pointing at host start, goal and obstacle arrays) and the
        prrtc_result array with its path buffers, built as numpy arrays with
        the C structs' layouts (no per-query ctypes work).  The path buffers
        (`paths`, path_capacity rows per query) are fresh memory: the first
        call that writes them also pays the operating system's zeroing of
        their pages (at 2048 rows of 7 floats per query, nearly every
        query's path lands on a page of its own: ~40 ms for 20 480 queries
        with 64 KB pages).  A caller
        that cares about the call's latency reuses the PreparedBatch or
        writes `paths` once beforehand."""
        rid = robot_id(robot)
        D, n = dof(rid), len(queries)
        trip = [q if isinstance(q, tuple) else (q.env, q.start, q.goal) for q in queries]
        starts = np.ascontiguousarray(np.asarray([s for _, s, _ in trip], np.float32).reshape(n, D))
        goals = None
        try:                                          # one goal (or k goals) per query: a single stack
            g = np.asarray([g for _, _, g in trip], np.float32)
            if g.ndim in (2, 3) and g.shape[0] == n and g.shape[-1] == D:
                ngoals = np.full(n, 1 if g.ndim == 2 else g.shape[1], np.int64)
                goals = np.ascontiguousarray(g.reshape(-1, D))
        except ValueError:                            # ragged goal lists
            pass
        if goals is None:
            goal_list = [np.asarray(g, np.float32).reshape(-1, D) for _, _, g in trip]
            goals = np.ascontiguousarray(np.concatenate(goal_list))
            ngoals = np.fromiter((len(g) for g in goal_list), np.int64, n)
        qs = np.zeros(n, _QUERY_DT)
        qs["start"] = starts.ctypes.data + 4 * D * np.arange(n, dtype=np.uint64)
        qs["goals"] = goals.ctypes.data + 4 * D * (np.cumsum(ngoals) - ngoals).astype(np.uint64)
        qs["num_goals"] = ngoals
        keep = [starts, goals]
        is_handle = np.fromiter((isinstance(e, EnvHandle) for e, _, _ in trip), bool, n)
        if is_handle.any():
            qs["env"][is_handle] = [e.handle.value for (e, _, _), h in zip(trip, is_handle) if h]
        plain = np.flatnonzero(~is_handle)
        if len(plain):
            descs = np.zeros(len(plain), _DESC_DT)
            envs = [trip[i][0] for i in plain]
            packed = all(type(e) is Environment for e in envs)   # float32, contiguous, [count, width] already
            for k in _ENV_KINDS:                       # one buffer per obstacle type, descriptors point into it
                arrs = [getattr(e, k) for e in envs] if packed else \
                    [np.asarray(getattr(e, k), np.float32) for e in envs]
                cnt = np.fromiter(map(len, arrs), np.int64, len(arrs))
                if cnt.sum():
                    buf = np.ascontiguousarray(np.concatenate(arrs))
                    keep.append(buf)
                    ptr = buf.ctypes.data + (buf.shape[1] * 4 * (np.cumsum(cnt) - cnt)).astype(np.uint64)
                    descs[k] = np.where(cnt > 0, ptr, 0)
                descs["num_" + k] = cnt
            keep.append(descs)
            qs["env_desc"][plain] = descs.ctypes.data + _DESC_DT.itemsize * np.arange(len(plain), dtype=np.uint64)
        paths = np.empty((n, path_capacity, D), np.float32)
        res = np.zeros(n, _RESULT_DT)
        res["path_capacity"] = path_capacity
        res["path"] = paths.ctypes.data + 4 * D * path_capacity * np.arange(n, dtype=np.uint64)
        return PreparedBatch(rid, qs, res, paths, keep)

    def solve_prepared(self, prep: "PreparedBatch", settings: BatchSettings | None = None) -> None:
        """The prrtc_solve_batch call itself on prepared host arrays; the
        answers land in prep.res and prep.paths."""
        s = settings if settings is not None else BatchSettings()
        self._check(lib().prrtc_solve_batch(self.handle, prep.rid, C.cast(C.c_void_p(prep.qs.ctypes.data), C.POINTER(_Query)),
                                            len(prep.qs), C.byref(s),
                                            C.cast(C.c_void_p(prep.res.ctypes.data), C.POINTER(_Result))))

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


@dataclass
class PreparedBatch:
    """prrtc_solve_batch's host arguments (Context.prepare_batch): the query
    and result arrays in the C layouts, the path buffers, and the host arrays
    they point into."""
    rid: int
    qs: np.ndarray
    res: np.ndarray
    paths: np.ndarray
    keep: list

    def results(self) -> list:
        res, paths = self.res, self.paths
        cols = {f: res[f].tolist() for f in ("solved", "path_rows", "start_tree_size", "goal_tree_size", "path_length",
                                             "iters", "cost", "wall_ns", "kernel_ns", "copy_ns", "status", "finish_ns",
                                             "samples")}
        return [PlannerResult(bool(cols["solved"][i]), paths[i, :cols["path_rows"][i]].copy(), cols["start_tree_size"][i],
                              cols["goal_tree_size"][i], cols["path_length"][i], cols["iters"][i], cols["cost"][i],
                              cols["wall_ns"][i], cols["kernel_ns"][i], cols["copy_ns"][i], cols["status"][i],
                              cols["finish_ns"][i], cols["samples"][i])
                for i in range(len(res))]


class Batch:
    """A prepared batch (prrtc_batch_create): run() solves every query in one
    persistent launch with inputs resident on the device; results() copies
    answers and paths back."""

    def __init__(self, ctx: "Context", robot, queries, settings: BatchSettings, path_capacity: int = 4096):
        self.ctx, self.rid = ctx, robot_id(robot)
        self.D = dof(self.rid)
        self.n = len(queries)
        self.path_capacity = path_capacity
        self._keep = []
        qs = (_Query * self.n)()
        for i, q in enumerate(queries):
            env, start, goals = q if isinstance(q, tuple) else (q.env, q.start, q.goal)
            start = np.ascontiguousarray(np.asarray(start, np.float32).reshape(self.D))
            goals = np.ascontiguousarray(np.asarray(goals, np.float32).reshape(-1, self.D))
            self._keep += [start, goals]
            if isinstance(env, EnvHandle):
                qs[i].env = env.handle
            else:
                d, keep = _env_desc(env)
                self._keep += [d, keep]
                qs[i].env_desc = C.cast(C.pointer(d), C.c_void_p)
            qs[i].start = start.ctypes.data
            qs[i].goals = goals.ctypes.data
            qs[i].num_goals = len(goals)
        self.settings = settings
        h = C.c_void_p()
        ctx._check(lib().prrtc_batch_create(ctx.handle, self.rid, qs, self.n, C.byref(settings), C.byref(h)))
        self.handle = h
        self._qs = qs

    def run(self):
        self.ctx._check(lib().prrtc_batch_run(self.ctx.handle, self.handle))

    def results(self) -> list:
        res = (_Result * self.n)()
        paths = np.empty((self.n, self.path_capacity, self.D), np.float32)
        for i in range(self.n):
            res[i].path_capacity = self.path_capacity
            res[i].path = paths[i].ctypes.data_as(C.POINTER(C.c_float))
        self.ctx._check(lib().prrtc_batch_results(self.ctx.handle, self.handle, res))
        return [PlannerResult(bool(r.solved), paths[i, :r.path_rows].copy(), r.start_tree_size, r.goal_tree_size,
                              r.path_length, r.iters, r.cost, r.wall_ns, r.kernel_ns, r.copy_ns, r.status, r.finish_ns,
                              r.samples)
                for i, r in enumerate(res)]

    def stats(self) -> dict:
        st = _BatchStats()
        self.ctx._check(lib().prrtc_batch_stats_get(self.ctx.handle, self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _BatchStats._fields_}

    def free(self):
        if getattr(self, "handle", None):
            lib().prrtc_batch_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.free()
        except Exception:
            pass


_ENV_KINDS = ("spheres", "capsules", "z_aligned_capsules", "cylinders", "cuboids", "z_aligned_cuboids")


def _numpy_dtype(struct) -> np.dtype:
    """A numpy structured dtype with a ctypes struct's field layout."""
    kinds = {C.c_void_p: "u8", C.c_int: "i4", C.c_uint32: "u4", C.c_uint64: "u8", C.c_int64: "i8", C.c_float: "f4"}
    names, formats, offsets = [], [], []
    for name, ctype in struct._fields_:
        names.append(name)
        offsets.append(getattr(struct, name).offset)
        formats.append("u8" if issubclass(ctype, C._Pointer) else kinds[ctype])
    return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": C.sizeof(struct)})


def _env_desc(env: Environment):
    keep, args = [], []
    for k in _ENV_KINDS:
        a = getattr(env, k)
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            a = np.ascontiguousarray(a, np.float32)
        keep.append(a)
        n = len(a)
        args += (a.ctypes.data if n else None, n)
    return EnvDesc(*args), keep


def _empty_like_device(t, shape, dtype: str):
    import torch
    return torch.empty(shape, dtype=getattr(torch, dtype), device=t.device)


_QUERY_DT = _numpy_dtype(_Query)
_DESC_DT = _numpy_dtype(EnvDesc)
_RESULT_DT = _numpy_dtype(_Result)
