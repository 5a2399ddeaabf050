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

    def prepare(self, env, q):
        """Builds the reference's Environment<float> for env on the device and
        returns (run, out): run() launches the checker once on the current
        stream over q (a host array or a CUDA tensor [n, dof]), writing
        verdicts (1 = free) into the CUDA tensor out [n]."""
        torch = self.torch
        q = q.contiguous() if hasattr(q, "data_ptr") else torch.from_numpy(_arr(q, self.dim)).cuda()
        assert q.dtype == torch.float32 and q.is_cuda and q.shape[-1] == self.dim
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

        def run():
            # q, arrs and scratch stay alive through this closure
            if n:
                self.launch(self.kname, (n + 127) // 128, 128,
                            [C.c_void_p(q.data_ptr()), C.c_longlong(n), C.c_int(self.dim),
                             C.c_void_p(scratch.data_ptr()), C.c_void_p(out.data_ptr())])
            return arrs
        return run, out[:n]

    def check(self, env, q) -> np.ndarray:
        """Reference verdicts (1 = free) for configurations q [n, dof]."""
        run, out = self.prepare(env, q)
        run()
        self.torch.cuda.synchronize()
        res = out.cpu().numpy()
        assert np.all(res <= 1), "reference GPU checker left verdicts unwritten"
        return res


class RefSampler(_Cubin):
    """pRRTC's own sampler (oracle/ref_planner_gpu.cu, which includes
    pRRTC.cu unmodified; `make -C oracle ref_sampler`): cuRAND states as
    pRRTC's init_rng makes them (pRRTC.cu:107-111, seed 1 as pRRTC::solve
    passes it), then the reference's halton_initialize / halton_next /
    scale_cfg for every lane."""

    PATH = HERE / "_ref" / "ref_sampler.cubin"
    INIT_RNG = "ref_init_rng"

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


class RefPlanner(_Cubin):
    """pRRTC's own planner kernel rrtc<Robot> (pRRTC.cu:305-602, in the cubin
    `make -C oracle ref_sampler` builds), driven the way pRRTC::solve drives
    it (pRRTC.cu:607-747): settings into d_settings, trees of -9999 nodes,
    cuRAND and Halton states, the start and goal roots, one launch of
    num_new_configs blocks of `granularity` threads, then the solved flag,
    tree sizes, cost and the two path halves read back and assembled goal
    first.

    That kernel writes tree slots past max_samples before it gives up
    (pRRTC.cu:451-453,535-537) and traces paths into a fixed
    path[2][5000] (pRRTC.cu:559-572) without bounds checks, so it runs here
    only under settings for which every write provably stays in bounds
    (`safe_rows` raises otherwise):
      * dynamic domain off, so every iteration of a block that does not
        return appends (no unbounded skip loop), and a block runs at most
        max_iters + 1 iterations (pRRTC.cu:343-346, 598);
      * an iteration appends at most 1 + E nodes to its block's tree, E =
        ceil(joint-box diameter / range) extension steps (every node lies in
        the box, so no connect distance exceeds its diameter);
      * so a tree holds at most R = roots + B (max_iters + 1) (1 + E) nodes,
        B = num_new_configs; the trees are allocated with R rows (more than
        max_samples if need be), and the parents arrays are zero-filled, so a
        parent read before its write lands is a valid index;
      * a traced half-path has at most R - 1 nodes, and R x dof <= 5000;
      * granularity a power of two <= 128 (the block's reduction reads
        sdata[tid + s] for every tid, pRRTC.cu:398-408, inside sdata[256])."""

    RRTC = {"sphere": "6Sphere", "panda": "5Panda", "fetch": "5Fetch", "baxter": "6Baxter"}
    MAX_PATH = 5000
    FLT_MAX = 3.4028234663852886e38

    def __init__(self, robot: str):
        r = self.RRTC[robot]
        self.k_rrtc = (f"_ZN5pRRTC4rrtcIN4ppln6robots{r}EEEvPPfPPiS5_PNS_11HaltonStateIT_EEP17curandStateXORWOW"
                       f"PNS1_9collision11EnvironmentIfEE")
        self.k_halton = f"_ZN5pRRTC11init_haltonIN4ppln6robots{r}EEEvPNS_11HaltonStateIT_EEP17curandStateXORWOW"
        super().__init__(RefSampler.PATH, [self.k_rrtc, self.k_halton, "ref_init_rng", "ref_reset", "ref_read",
                                           "ref_env_build", "ref_env_bytes", "ref_curand_state_bytes"])
        torch = self.torch
        self.robot = robot
        self.dim = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]
        sz = torch.zeros(5, dtype=torch.int64, device="cuda")
        self.launch("ref_curand_state_bytes", 1, 1, [C.c_void_p(sz.data_ptr())])
        es = torch.zeros(5, dtype=torch.int64, device="cuda")
        self.launch("ref_env_bytes", 1, 1, [C.c_void_p(es.data_ptr())])
        torch.cuda.synchronize()
        sz = [int(v) for v in sz.cpu()]
        self.rng_bytes = sz[0]
        self.halton_bytes = sz[1 + ["sphere", "panda", "fetch", "baxter"].index(robot)]
        self.env_sizes = [int(v) for v in es.cpu()]
        cu = self._driver()
        cu.cuModuleGetGlobal_v2.restype = C.c_int
        cu.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        cu.cuMemcpyHtoD_v2.restype = C.c_int
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        self.d_settings, nbytes = C.c_uint64(), C.c_size_t()
        self._ok(cu.cuModuleGetGlobal_v2(C.byref(self.d_settings), C.byref(nbytes), self.mod,
                                         b"_ZN5pRRTC10d_settingsE"), "d_settings")
        self.settings_bytes = nbytes.value

    @classmethod
    def available(cls) -> bool:
        return RefSampler.PATH.exists()

    @staticmethod
    def safe_rows(robot: str, settings, num_goals: int) -> int:
        """Tree rows that hold every node the kernel can append under these
        settings; raises ValueError when they are not provably safe."""
        import math
        from prrtc_gb300 import scenes
        dim = {"sphere": 3, "panda": 7, "fetch": 8, "baxter": 14}[robot]
        if settings.dynamic_domain:
            raise ValueError("dynamic domain: a block may skip iterations without bound")
        g = settings.granularity
        if g < 1 or g > 128 or g & (g - 1):
            raise ValueError("granularity must be a power of two <= 128")
        diam = math.sqrt(sum(s * s for s in scenes.LIMITS[robot][0])) * (1 + 1e-6)
        ext = math.ceil(diam / settings.range)
        rows = max(1, num_goals) + settings.num_new_configs * (settings.max_iters + 1) * (1 + ext)
        if rows * dim > RefPlanner.MAX_PATH:
            raise ValueError(f"a traced path could need {rows * dim} floats > {RefPlanner.MAX_PATH}")
        return max(rows, settings.max_samples)

    def solve(self, start, goals, env, settings) -> dict:
        torch = self.torch
        D = self.dim
        start = _arr(start, D)
        goals = _arr(goals, D)
        ng = len(goals)
        rows = self.safe_rows(self.robot, settings, ng)
        B, g = settings.num_new_configs, settings.granularity
        s_bytes = C.string_at(C.addressof(settings), C.sizeof(settings))
        assert len(s_bytes) == self.settings_bytes == 44
        self._ok(self._driver().cuMemcpyHtoD_v2(self.d_settings.value, s_bytes, len(s_bytes)), "settings")
        dev = "cuda"
        nodes = [torch.full((rows * D,), -9999.0, dtype=torch.float32, device=dev) for _ in range(2)]
        parents = [torch.zeros(rows, dtype=torch.int32, device=dev) for _ in range(2)]
        radii = [torch.zeros(rows, dtype=torch.float32, device=dev) for _ in range(2)]
        radii[0][0] = self.FLT_MAX
        radii[1][:ng] = self.FLT_MAX
        nodes[0][:D] = torch.from_numpy(start.reshape(-1)).to(dev)
        nodes[1][:ng * D] = torch.from_numpy(goals.reshape(-1)).to(dev)
        parents[1][:ng] = torch.arange(ng, dtype=torch.int32, device=dev)
        ptrs = [torch.tensor([t[0].data_ptr(), t[1].data_ptr()], dtype=torch.int64, device=dev)
                for t in (nodes, parents, radii)]
        nrng = B * D
        rng = torch.zeros(nrng * self.rng_bytes + 256, dtype=torch.uint8, device=dev)
        halton = torch.zeros(B * self.halton_bytes + 256, dtype=torch.uint8, device=dev)
        self.launch("ref_init_rng", (nrng + 63) // 64, 64, [C.c_void_p(rng.data_ptr()), C.c_ulong(1), C.c_int(nrng)])
        self.launch(self.k_halton, (B + 63) // 64, 64, [C.c_void_p(halton.data_ptr()), C.c_void_p(rng.data_ptr())])
        self.launch("ref_reset", 1, 1, [C.c_int(1), C.c_int(ng)])
        arrs = [torch.from_numpy(_arr(a, k)).to(dev) for a, k in
                ((env.spheres, 4), (env.capsules, 8), (env.z_aligned_capsules, 8), (env.cuboids, 15),
                 (env.z_aligned_cuboids, 15))]
        per = [self.env_sizes[1], self.env_sizes[2], self.env_sizes[2], self.env_sizes[3], self.env_sizes[3]]
        nbytes = (self.env_sizes[0] + 255) // 256 * 256 + sum((p * len(a) + 255) // 256 * 256 for p, a in zip(per, arrs))
        scratch = torch.zeros(nbytes + 256, dtype=torch.uint8, device=dev)
        eargs = [C.c_void_p(scratch.data_ptr())]
        for a in arrs:
            eargs += [C.c_void_p(a.data_ptr() if len(a) else 0), C.c_int(len(a))]
        self.launch("ref_env_build", 1, 1, eargs)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        self.launch(self.k_rrtc, B, g, [C.c_void_p(p.data_ptr()) for p in ptrs] +
                    [C.c_void_p(halton.data_ptr()), C.c_void_p(rng.data_ptr()), C.c_void_p(scratch.data_ptr())])
        ev1.record()
        ints = torch.zeros(7, dtype=torch.int32, device=dev)
        cost = torch.zeros(1, dtype=torch.float32, device=dev)
        path = torch.zeros(2 * self.MAX_PATH, dtype=torch.float32, device=dev)
        self.launch("ref_read", 1, 1, [C.c_void_p(ints.data_ptr()), C.c_void_p(cost.data_ptr()),
                                       C.c_void_p(path.data_ptr())])
        torch.cuda.synchronize()
        ii = [int(v) for v in ints.cpu()]
        out = {"solved": ii[0] == 1, "start_tree_size": ii[1], "goal_tree_size": ii[2], "iters": ii[6],
               "kernel_ms": ev0.elapsed_time(ev1), "cost": float(cost.item()), "path": None}
        if out["solved"]:
            p = path.cpu().numpy().reshape(2, self.MAX_PATH)
            n0, n1 = ii[3], ii[4]
            rows_out = [goals[ii[5]]]
            rows_out += [p[1, i * D:(i + 1) * D] for i in range(n1 - 1, -1, -1)]
            rows_out += [p[0, i * D:(i + 1) * D] for i in range(n0)]
            rows_out.append(start[0])
            out["path"] = np.stack(rows_out).astype(np.float32)
            out["path_length"] = n0 + n1
        return out
