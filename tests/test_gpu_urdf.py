"""Robot-model compiler on the GPU: checkers generated from URDF models run on
the device and agree with the models' float64 semantics.

Two robots go through urdf.build_model -> codegen -> nvcc (sm_103a): the
4-joint test arm of test_urdf.py (fixed, revolute, continuous and prismatic
joints) and Panda's fitted model written out as a URDF and read back.  Each
generated checker (fkcc_validate, the straight-line form codegen emits for
robots outside the table-form list) runs on 10^5 seeded configurations per
scene; its verdicts must equal the float64 verdict of the same model
(scenes.clearance_model: free when no leaf sphere penetrates an obstacle and
no listed leaf pair penetrates) except within 1e-5 m of contact."""
import ctypes as C
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NEAR = 1e-5


def pack_records(env) -> np.ndarray:
    """The device's packed environment (float4 records, device_common.cuh)."""
    recs = [np.asarray(env.spheres, np.float32).reshape(-1, 4)]
    for caps in (env.capsules, env.z_aligned_capsules):
        c = np.asarray(caps, np.float32).reshape(-1, 8)
        r = np.empty((len(c), 2, 4), np.float32)
        r[:, 0, :3], r[:, 0, 3], r[:, 1, :3], r[:, 1, 3] = c[:, 0:3], c[:, 6], c[:, 3:6], c[:, 7]
        recs.append(r.reshape(-1, 4))
    for cubs in (env.cuboids, env.z_aligned_cuboids):
        c = np.asarray(cubs, np.float32).reshape(-1, 15)
        r = np.zeros((len(c), 4, 4), np.float32)
        r[:, 0, :3], r[:, 0, 3] = c[:, 0:3], c[:, 12]
        r[:, 1, :3], r[:, 1, 3] = c[:, 3:6], c[:, 13]
        r[:, 2, :3], r[:, 2, 3] = c[:, 6:9], c[:, 14]
        r[:, 3, :3] = c[:, 9:12]
        recs.append(r.reshape(-1, 4))
    out = np.concatenate(recs)
    return out if len(out) else np.zeros((1, 4), np.float32)


KERNEL = r"""
#include "device_common.cuh"
{includes}
template <int D, class F>
__global__ void k_check(const float4 *env, prrtc::EnvCounts nc, const float *q, long n, unsigned char *out, F f)
{{
    prrtc::CheckCtx ctx{{{{env, nc}}, 0.0f, nullptr}};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {{
        float cfg[D];
        for (int d = 0; d < D; d++) cfg[d] = q[i * D + d];
        out[i] = f(cfg, ctx) ? 1 : 0;
    }}
}}
{wrappers}
"""

WRAPPER = r"""
struct Call_{name} {{
    __device__ bool operator()(const float *c, prrtc::CheckCtx &ctx) const {{ return prrtc::gen_{name}::fkcc_validate(c, ctx); }}
}};
extern "C" int check_{name}(const float4 *env, int ns, int nc, int nzc, int ncb, int nzb, const float *q, long n,
                            unsigned char *out)
{{
    k_check<prrtc::gen_{name}::kDof><<<152 * 4, 128>>>(env, prrtc::EnvCounts{{ns, nc, nzc, ncb, nzb}}, q, n, out,
                                                      Call_{name}{{}});
    const cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? (int)cudaGetLastError() : (int)e;
}}
"""


@pytest.fixture(scope="module")
def compiled(tmp_path_factory, ctx):
    import prrtc_gb300.build as b
    from prrtc_gb300.robots import codegen, urdf
    from test_urdf import ARM, SPHERES, panda_round_trip
    d = tmp_path_factory.mktemp("urdf_gpu")
    models = {"arm": urdf.build_model(ARM, SPHERES, "arm"), "panda_rt": panda_round_trip(reference_pairs_only=True)[0]}
    for name, m in models.items():
        (d / f"{name}_model.h").write_text(
            codegen.emit_c_tables(m).replace('#include "model_types.h"', '#include "robots/model_types.h"'))
        (d / f"{name}_fkcc.cuh").write_text(codegen.emit_cuda_checker(m))
    includes = "\n".join(f'#include "{n}_model.h"\n#include "{n}_fkcc.cuh"' for n in models)
    wrappers = "\n".join(WRAPPER.format(name=n) for n in models)
    (d / "k.cu").write_text(KERNEL.format(includes=includes, wrappers=wrappers))
    so = d / "liburdf_checkers.so"
    subprocess.run([b.NVCC, *b.ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared",
                    f"-I{b.CSRC}", f"-I{d}", str(d / "k.cu"), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    for n in models:
        f = getattr(L, f"check_{n}")
        f.restype = C.c_int
        f.argtypes = [C.c_void_p] + [C.c_int] * 5 + [C.c_void_p, C.c_long, C.c_void_p]
    return L, models


def run(L, name, env, q):
    import torch
    rec = torch.from_numpy(pack_records(env)).cuda()
    qd = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
    out = torch.full((len(q),), 7, dtype=torch.uint8, device="cuda")
    counts = [len(env.spheres), len(env.capsules), len(env.z_aligned_capsules), len(env.cuboids),
              len(env.z_aligned_cuboids)]
    assert getattr(L, f"check_{name}")(rec.data_ptr(), *counts, qd.data_ptr(), len(q), out.data_ptr()) == 0
    return out.cpu().numpy()


CASES = [("arm", "mixed", 1), ("arm", "mixed", 2), ("panda_rt", "tabletop", 3), ("panda_rt", "shelf", 4)]


@pytest.mark.parametrize("name,kind,seed", CASES)
def test_urdf_checker_matches_model(compiled, name, kind, seed):
    from prrtc_gb300 import scenes
    L, models = compiled
    m = models[name]
    if kind == "mixed":
        env = scenes.mixed_scene(seed, 12, lo=(0.2, -0.5, 0.0), hi=(0.8, 0.5, 0.8), n_zaligned=4)
    elif kind == "tabletop":
        env = scenes.tabletop_scene(seed, n_zaligned=8)
    else:
        env = scenes.shelf_scene(seed, n_zaligned=6)
    lo, hi = np.array(m["limits"]["lower"]), np.array(m["limits"]["upper"])
    q = (np.random.default_rng(seed).random((100_000, m["dof"])) * (hi - lo) + lo).astype(np.float32)
    got = run(L, name, env, q)
    cl = scenes.clearance_model(m, env, q.astype(np.float64))
    want = (cl >= 0).astype(np.uint8)
    bad = np.flatnonzero(got != want)
    near = int((np.abs(cl) < NEAR).sum())
    print(f"{name}/{kind}: 1e5 configs, free {want.mean():.3f}, mismatches {len(bad)}, near-contact {near}")
    assert 0.02 < want.mean() < 0.98
    assert np.all(np.abs(cl[bad]) < NEAR)
