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
    """make the oracle (and the reference checker), holding a file lock so
    that processes starting together build once."""
    import fcntl
    with open(HERE / ".build.lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            subprocess.run(["make", "-s", "-C", str(HERE)] + (["ref"] if ref else []), check=True)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


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
        self.L.oracle_halton.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
        self.L.oracle_nearest.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        self.L.oracle_dd_apply.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float]
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

    def halton(self, bases16, steps, scale, offset):
        """halton_next per lane from bases16 [lanes, 16]: (raw, scaled), each [lanes, steps, dof]."""
        D = len(scale)
        b = np.ascontiguousarray(np.asarray(bases16, np.float32).reshape(-1, 16))
        sc = np.ascontiguousarray(np.asarray(scale, np.float32))
        of = np.ascontiguousarray(np.asarray(offset, np.float32))
        raw = np.empty((len(b), steps, D), np.float32)
        cfg = np.empty_like(raw)
        assert self.L.oracle_halton(D, b.ctypes.data, len(b), steps, sc.ctypes.data, of.ctypes.data, raw.ctypes.data,
                                    cfg.ctypes.data) == 0
        return raw, cfg

    def nearest(self, nodes, q):
        """(index, squared distance) of the nearest of nodes [count, dof] to each row of q."""
        nodes = np.ascontiguousarray(np.asarray(nodes, np.float32))
        q = np.ascontiguousarray(np.asarray(q, np.float32).reshape(-1, nodes.shape[1]))
        oi = np.empty(len(q), np.int32)
        od = np.empty(len(q), np.float32)
        assert self.L.oracle_nearest(nodes.shape[1], nodes.ctypes.data, len(nodes), q.ctypes.data, len(q),
                                     oi.ctypes.data, od.ctypes.data) == 0
        return oi, od

    def dd_apply(self, radii, ops, alpha, radius0, rmin):
        """Radii after applying ops [n, k] (0 grow, 1 shrink) in order."""
        r = np.array(radii, np.float32)
        ops = np.ascontiguousarray(np.asarray(ops, np.uint8).reshape(len(r), -1))
        assert self.L.oracle_dd_apply(r.ctypes.data, len(r), ops.ctypes.data, ops.shape[1], alpha, radius0, rmin) == 0
        return r

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


class _Cubin:
    """A cubin built here from the reference sources, loaded through the CUDA
    driver API into the current (torch's primary) context; kernels launch on
    torch's current stream with device pointers from torch tensors."""

    _CU = None

    def __init__(self, path: Path, names):
        import torch
        self.torch = torch
        torch.zeros(1, device="cuda")          # make torch's primary context current
        cu = self._driver()
        self.mod = C.c_void_p()
        self._ok(cu.cuModuleLoad(C.byref(self.mod), str(path).encode()), f"cuModuleLoad {path.name}")
        self.fn = {}
        for name in names:
            f = C.c_void_p()
            self._ok(cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f

    @classmethod
    def _driver(cls):
        if cls._CU is None:
            cu = C.CDLL("libcuda.so.1")
            for f in ("cuModuleLoad", "cuModuleGetFunction", "cuLaunchKernel"):
                getattr(cu, f).restype = C.c_int
            cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
            cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
            cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                          C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
            cls._CU = cu
        return cls._CU

    @staticmethod
    def _ok(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def launch(self, name, grid, block, args):
        stream = self.torch.cuda.current_stream().cuda_stream
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._ok(self._driver().cuLaunchKernel(self.fn[name], grid, 1, 1, block, 1, 1, 0, C.c_void_p(stream), ptrs,
                                               None), f"cuLaunchKernel {name}")


class RefGpuChecker(_Cubin):
    """pRRTC's own GPU checker: fkcc<Robot> (utils.cuh:326-327) in the harness
    kernels of oracle/ref_fkcc_gpu.cu, one sm_103a cubin per robot built by
    `make -C oracle ref_gpu`.  Each check builds the reference's
    Environment<float> on the device, then runs one configuration per
    thread."""

    def __init__(self, robot: str):
        self.kname = f"ref_fkcc_gpu_{REF_NAMES[robot]}"
        super().__init__(self.path(robot), (self.kname, "ref_env_build", "ref_env_bytes"))
        torch = self.torch
        self.dim = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]
        sizes = torch.zeros(5, dtype=torch.int64, device="cuda")
        self.launch("ref_env_bytes", 1, 1, [C.c_void_p(sizes.data_ptr())])
        torch.cuda.synchronize()
        self.sizes = [int(v) for v in sizes.cpu()]   # Environment, Sphere, Capsule, Cuboid sizes; alignment
        assert self.sizes[4] <= 256

    @staticmethod
    def path(robot: str) -> Path:
        return HERE / "_ref" / f"ref_fkcc_gpu_{REF_NAMES[robot]}.cubin"

    @classmethod
    def available(cls, robot: str) -> bool:
        return cls.path(robot).exists()

    def check(self, env, q) -> np.ndarray:
        """Reference verdicts (1 = free) for configurations q [n, dof]."""
        torch = self.torch
        q = torch.from_numpy(_arr(q, self.dim)).cuda()
        arrs = [torch.from_numpy(_arr(a, k)).cuda() for a, k in
                ((env.spheres, 4), (env.capsules, 8), (env.z_aligned_capsules, 8), (env.cuboids, 15),
                 (env.z_aligned_cuboids, 15))]
        per = [self.sizes[1], self.sizes[2], self.sizes[2], self.sizes[3], self.sizes[3]]

        def r256(b):
            return (b + 255) // 256 * 256

        nbytes = r256(self.sizes[0]) + sum(r256(p * len(a)) for p, a in zip(per, arrs))
        scratch = torch.zeros(nbytes + 256, dtype=torch.uint8, device="cuda")
        assert scratch.data_ptr() % 256 == 0
        eargs = [C.c_void_p(scratch.data_ptr())]
        for a in arrs:
            eargs += [C.c_void_p(a.data_ptr() if len(a) else 0), C.c_int(len(a))]
        self.launch("ref_env_build", 1, 1, eargs)
        n = len(q)
        out = torch.full((max(n, 1),), 255, dtype=torch.uint8, device="cuda")
        if n:
            self.launch(self.kname, (n + 127) // 128, 128,
                        [C.c_void_p(q.data_ptr()), C.c_longlong(n), C.c_int(self.dim),
                         C.c_void_p(scratch.data_ptr()), C.c_void_p(out.data_ptr())])
        torch.cuda.synchronize()
        res = out[:n].cpu().numpy()
        assert np.all(res <= 1), "reference GPU checker left verdicts unwritten"
        return res


class RefSampler(_Cubin):
    """pRRTC's own sampler (oracle/ref_planner_gpu.cu, which includes
    pRRTC.cu unmodified; `make -C oracle ref_sampler`): the reference's
    init_rng kernel (pRRTC.cu:107-111, seed 1 as pRRTC::solve passes it),
    then halton_initialize / halton_next / scale_cfg for every lane."""

    PATH = HERE / "_ref" / "ref_sampler.cubin"
    INIT_RNG = "_ZN6pRRTC8init_rngEP17curandStateXORWOWmi"   # pRRTC::init_rng(curandState*, unsigned long, int)

    def __init__(self):
        super().__init__(self.PATH, [self.INIT_RNG, "ref_curand_state_bytes"] +
                         [f"ref_halton_{r}" for r in REF_NAMES.values()])
        torch = self.torch
        sz = torch.zeros(1, dtype=torch.int64, device="cuda")
        self.launch("ref_curand_state_bytes", 1, 1, [C.c_void_p(sz.data_ptr())])
        torch.cuda.synchronize()
        self.state_bytes = int(sz.item())

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()

    def run(self, robot: str, lanes: int, steps: int):
        """(bases [lanes, dof], raw [lanes, steps, dof], scaled [lanes, steps, dof])."""
        torch = self.torch
        D = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]
        states = torch.zeros(lanes * self.state_bytes + 256, dtype=torch.uint8, device="cuda")
        self.launch(self.INIT_RNG, (lanes + 63) // 64, 64,
                    [C.c_void_p(states.data_ptr()), C.c_ulong(1), C.c_int(lanes)])
        bases = torch.empty((lanes, D), dtype=torch.float32, device="cuda")
        raw = torch.empty((lanes, steps, D), dtype=torch.float32, device="cuda")
        cfg = torch.empty_like(raw)
        self.launch(f"ref_halton_{REF_NAMES[robot]}", (lanes + 63) // 64, 64,
                    [C.c_void_p(states.data_ptr()), C.c_void_p(bases.data_ptr()), C.c_void_p(raw.data_ptr()),
                     C.c_void_p(cfg.data_ptr()), C.c_int(lanes), C.c_int(steps)])
        torch.cuda.synchronize()
        return bases.cpu().numpy(), raw.cpu().numpy(), cfg.cpu().numpy()
