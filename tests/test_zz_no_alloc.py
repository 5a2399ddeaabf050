"""prrtc_validate_configs_noalloc: the allocation-free checking entry point
gives the same verdicts as prrtc_validate_configs, call after call.

It exists for callers that cannot allocate device memory (deadline-bound
control loops, processes whose device memory belongs to another runtime);
its only device storage is a fixed array inside the library, reused by every
call.  This file is collected last so that a failure here never hides the
other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc():
    from prrtc_gb300 import api
    f = api.lib().prrtc_validate_configs_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.POINTER(api.EnvDesc), C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    return f


def test_noalloc_matches_validate_configs_two_calls():
    import torch
    import prrtc_gb300.build as b
    b.build()
    from prrtc_gb300 import Context, api, scenes
    f = _noalloc()
    ctx = Context(0)   # the existing entry point, for comparison
    cases = [("panda", scenes.shelf_scene(3), 0), ("fetch", scenes.mixed_scene(5, 40), 1)]
    for robot, env, seed in cases:   # two calls in a row, different scenes and robots
        sc, off = (np.array(v) for v in scenes.LIMITS[robot])
        q = (np.random.default_rng(seed).random((50000, len(sc))) * sc + off).astype(np.float32)
        qd = torch.from_numpy(q).cuda()
        out = torch.full((len(q),), 7, dtype=torch.uint8, device="cuda")
        d, keep = api._env_desc(env)
        st = f(api.robot_id(robot), C.byref(d), qd.data_ptr(), len(q), out.data_ptr(), None)
        torch.cuda.synchronize()
        assert st == 0
        ref = ctx.validate_configs(robot, env, q)
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
    ctx.close()


def test_noalloc_rejects_environment_beyond_the_fixed_array():
    import torch
    from prrtc_gb300 import api
    from prrtc_gb300.env import Environment
    f = _noalloc()
    big = Environment(cuboids=np.zeros((800, 15), np.float32))   # 12800 packed floats > PRRTC_MAX_ENV_FLOATS
    d, keep = api._env_desc(big)
    qd = torch.zeros((4, 7), dtype=torch.float32, device="cuda")
    out = torch.zeros(4, dtype=torch.uint8, device="cuda")
    assert f(api.robot_id("panda"), C.byref(d), qd.data_ptr(), 4, out.data_ptr(), None) == 1   # PRRTC_EINVAL
