"""Context.prepare_batch: the prrtc_query / prrtc_result arrays it builds for
prrtc_solve_batch point at the right host data (read back through the
pointers, no GPU): starts, goal lists of different lengths, every obstacle
list of every query's environment descriptor (empty lists as null), and one
path buffer per result."""
import ctypes as C

import numpy as np


def floats_at(addr, n):
    return np.frombuffer(C.string_at(int(addr), 4 * n), np.float32)


def test_prepared_arrays_point_at_the_host_data():
    from prrtc_gb300 import Context, Environment
    from prrtc_gb300.api import EnvDesc, _ENV_KINDS
    rng = np.random.default_rng(0)
    envs = [Environment(spheres=rng.random((3, 4)), cuboids=rng.random((2, 15))),
            Environment(),
            Environment(capsules=rng.random((1, 8)), z_aligned_cuboids=rng.random((4, 15)), spheres=rng.random((1, 4)))]
    starts = [rng.random(7).astype(np.float32) for _ in envs]
    goals = [rng.random((k, 7)).astype(np.float32) for k in (1, 3, 2)]
    ctx = Context.__new__(Context)   # marshalling only: no device context needed
    ctx.handle = None
    prep = ctx.prepare_batch("panda", list(zip(envs, starts, goals)), path_capacity=16)
    assert len(prep.qs) == 3 and prep.paths.shape == (3, 16, 7)
    for i, (e, s, g) in enumerate(zip(envs, starts, goals)):
        q = prep.qs[i]
        np.testing.assert_array_equal(floats_at(q["start"], 7), s)
        assert q["num_goals"] == len(g)
        np.testing.assert_array_equal(floats_at(q["goals"], 7 * len(g)).reshape(-1, 7), g)
        assert q["env"] == 0
        d = EnvDesc.from_address(int(q["env_desc"]))
        for k in _ENV_KINDS:
            a = getattr(e, k)
            assert getattr(d, "num_" + k) == len(a), (i, k)
            if len(a):
                np.testing.assert_array_equal(floats_at(getattr(d, k), a.size).reshape(a.shape), a)
            else:
                assert not getattr(d, k), (i, k)
        r = prep.res[i]
        assert r["path_capacity"] == 16 and int(r["path"]) == prep.paths[i].ctypes.data
