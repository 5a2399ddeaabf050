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


def test_noalloc_queued_calls_on_one_stream_and_empty_scene():
    """Two calls queued back to back on one non-default stream, with a single
    synchronise after both (the second reuses the fixed array while the first
    may still be running, ordered by the stream), then a call with no
    obstacles at all.  Each verdict buffer matches prrtc_validate_configs,
    and the first also matches the oracle outside the near-contact bucket."""
    import sys
    import torch
    import prrtc_gb300.build as b
    b.build()
    from conftest import ROOT
    sys.path.insert(0, str(ROOT / "oracle"))
    from pyoracle import OracleLib
    from prrtc_gb300 import Context, api, scenes
    from prrtc_gb300.env import Environment
    f = _noalloc()
    ctx = Context(0)
    envs = [scenes.tabletop_scene(7, n_zaligned=8), scenes.shelf_scene(8, n_zaligned=6), Environment()]
    sc, off = (np.array(v) for v in scenes.LIMITS["panda"])
    qs = [(np.random.default_rng(20 + i).random((30000, 7)) * sc + off).astype(np.float32) for i in range(3)]
    st = torch.cuda.Stream()
    outs, keep = [], []
    with torch.cuda.stream(st):
        qd = [torch.from_numpy(q).cuda() for q in qs]
        for i in range(2):
            out = torch.full((len(qs[i]),), 7, dtype=torch.uint8, device="cuda")
            d, k = api._env_desc(envs[i])
            keep.append((d, k))
            assert f(api.robot_id("panda"), C.byref(d), qd[i].data_ptr(), len(qs[i]), out.data_ptr(),
                     C.c_void_p(st.cuda_stream)) == 0
            outs.append(out)
    st.synchronize()
    d, k = api._env_desc(envs[2])
    out = torch.full((len(qs[2]),), 7, dtype=torch.uint8, device="cuda")
    assert f(api.robot_id("panda"), C.byref(d), qd[2].data_ptr(), len(qs[2]), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    outs.append(out)
    for env, q, o in zip(envs, qs, outs):
        np.testing.assert_array_equal(o.cpu().numpy(), ctx.validate_configs("panda", env, q))
    ref, margin = OracleLib().check("panda", envs[0], qs[0], margin=True)
    bad = np.flatnonzero(outs[0].cpu().numpy() != ref)
    assert (margin[bad] < 1e-5).all()
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


def test_noalloc_refuses_stream_capture():
    """The call copies its obstacles from a library host array when it runs,
    so it is not capturable into a CUDA graph.  While the stream is being
    captured it must return PRRTC_EINVAL and leave the stream alone: the
    capture ends cleanly, and a replay runs only the work captured around
    the refused call."""
    import torch
    from prrtc_gb300 import api, scenes
    f = _noalloc()
    env = scenes.shelf_scene(3)
    sc, off = (np.array(v) for v in scenes.LIMITS["panda"])
    q = (np.random.default_rng(9).random((4096, 7)) * sc + off).astype(np.float32)
    qd = torch.from_numpy(q).cuda()
    out = torch.full((len(q),), 7, dtype=torch.uint8, device="cuda")
    d, keep = api._env_desc(env)
    s = torch.cuda.Stream()
    # an ordinary call first, on the same stream (the per-device setup)
    assert f(api.robot_id("panda"), C.byref(d), qd.data_ptr(), len(q), out.data_ptr(), C.c_void_p(s.cuda_stream)) == 0
    s.synchronize()
    first = out.clone()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        status = f(api.robot_id("panda"), C.byref(d), qd.data_ptr(), len(q), out.data_ptr(),
                   C.c_void_p(s.cuda_stream))
        out.add_(0)   # captured work beside the refused call, so the graph is not empty
    assert status == 1   # PRRTC_EINVAL
    out.fill_(7)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    assert (out == 7).all()   # the replay did not write verdicts: nothing of the call was recorded
    out.copy_(first)
    assert f(api.robot_id("panda"), C.byref(d), qd.data_ptr(), len(q), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), first.cpu().numpy())
