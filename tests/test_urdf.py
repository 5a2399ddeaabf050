"""Robot-model compiler front end (URDF + spheres -> model): kinematics against
direct URDF semantics, a round trip through Panda's fitted model, and the
generated checker compiling for sm_103a."""
import math
import shutil
import subprocess

import numpy as np
import pytest

ARM = """<robot name="arm">
  <link name="base"/> <link name="l1"/> <link name="l1b"/> <link name="l2"/> <link name="l3"/> <link name="tool"/>
  <joint name="j1" type="revolute"><parent link="base"/><child link="l1"/>
    <origin xyz="0 0 0.3" rpy="0 0 0.4"/><axis xyz="0 0 1"/><limit lower="-2.9" upper="2.9"/></joint>
  <joint name="f1" type="fixed"><parent link="l1"/><child link="l1b"/><origin xyz="0.05 0 0.1" rpy="0.3 0 0"/></joint>
  <joint name="j2" type="revolute"><parent link="l1b"/><child link="l2"/>
    <origin xyz="0 0.02 0.2" rpy="0.1 -0.2 0.3"/><axis xyz="0 1 0"/><limit lower="-1.5" upper="1.5"/></joint>
  <joint name="j3" type="continuous"><parent link="l2"/><child link="l3"/>
    <origin xyz="0.4 0 0" rpy="0 0.5 0"/><axis xyz="0.3 -0.5 0.8"/></joint>
  <joint name="j4" type="prismatic"><parent link="l3"/><child link="tool"/>
    <origin xyz="0.2 0 0" rpy="0 0 0"/><axis xyz="-1 0 0"/><limit lower="0" upper="0.1"/></joint>
</robot>"""
SPHERES = {"base": [[0, 0, 0.1, 0.12]], "l1": [[0, 0, 0.05, 0.08], [0.02, 0, 0.15, 0.06]],
           "l1b": [[0, 0.03, 0.05, 0.05]], "l2": [[0.1, 0, 0, 0.05], [0.2, 0, 0, 0.05], [0.3, 0, 0, 0.04]],
           "l3": [[0.05, 0.01, 0, 0.04], [0.15, 0, 0.01, 0.04]], "tool": [[0.0, 0, 0, 0.03], [0.05, 0, 0, 0.02]]}


def model_centres(m, q):
    from prrtc_gb300.robots.extract import model_sphere_centres
    return model_sphere_centres(m, q[None, :])[:, 0, :]


def test_arm_kinematics_match_urdf():
    from prrtc_gb300.robots import urdf
    m = urdf.build_model(ARM, SPHERES, "arm")
    assert m["dof"] == 4 and [j["type"] for j in m["joints"]] == ["revolute", "revolute", "revolute", "prismatic"]
    assert m["limits"]["lower"][2] == -math.pi and m["limits"]["upper"][3] == 0.1
    rng = np.random.default_rng(0)
    leaves = [i for g in m["env_groups"] for i in g["leaves"]]
    for _ in range(20):
        q = rng.uniform(-2, 2, 4)
        want = np.concatenate([np.array(v) for v in urdf.urdf_sphere_centres(ARM, SPHERES, q).values()])
        got = model_centres(m, q)[leaves]
        np.testing.assert_allclose(got, want, atol=1e-12)


def test_arm_groups():
    """Joined links and links on one rigid body are never checked together."""
    from prrtc_gb300.robots import urdf
    m = urdf.build_model(ARM, SPHERES, "arm")
    labels = {g["label"] for g in m["self_groups"]}
    assert "base vs. l1" not in labels and "l1 vs. l1b" not in labels and "l2 vs. l3" not in labels
    assert "base vs. l2" in labels and "l1 vs. tool" in labels
    for g in m["env_groups"]:   # a multi-sphere link's gate bounds its leaves at q = 0
        if g["gate"] >= 0:
            c = model_centres(m, np.zeros(4))
            gs = m["spheres"][g["gate"]]
            for i in g["leaves"]:
                assert np.linalg.norm(c[i] - c[g["gate"]]) + m["spheres"][i]["r"] <= gs["r"] + 1e-12


def rpy_of(R):
    """Inverse of R = Rz(y) Ry(p) Rx(r)."""
    if abs(R[2, 0]) < 1 - 1e-12:
        return math.atan2(R[2, 1], R[2, 2]), -math.asin(R[2, 0]), math.atan2(R[1, 0], R[0, 0])
    p = -math.copysign(math.pi / 2, R[2, 0])
    return 0.0, p, math.atan2(-R[0, 1], R[1, 1])


def panda_round_trip(reference_pairs_only: bool = False):
    """Panda's fitted model written out as a URDF (joint origins from F, axis
    z) and read back: (the model built from the URDF, Panda's model, the
    index of each URDF-model leaf in Panda's sphere list).  With
    reference_pairs_only, link pairs that pRRTC's Panda model never checks
    against each other are passed as allowed (as an SRDF's disabled
    collisions would be), so only the link pairs pRRTC checks are checked,
    and only pRRTC's leaf spheres become collision geometry."""
    from prrtc_gb300.robots import urdf
    from prrtc_gb300.robots.codegen import load_model
    pm = load_model("panda")
    link = {-1: "world"} | {j["q"]: f"link{j['q']}" for j in pm["joints"]}
    parts = ['<robot name="p"><link name="world"/>']
    for j in pm["joints"]:
        F = np.array(j["F"])
        r, p, y = rpy_of(F[:, :3])
        np.testing.assert_allclose(urdf.rpy_matrix(r, p, y), F[:, :3], atol=1e-12)
        parts.append(f'<link name="{link[j["q"]]}"/><joint name="j{j["q"]}" type="{j["type"]}">'
                     f'<parent link="{link[j["parent"]]}"/><child link="{link[j["q"]]}"/>'
                     f'<origin xyz="{float(F[0, 3])!r} {float(F[1, 3])!r} {float(F[2, 3])!r}" rpy="{r!r} {p!r} {y!r}"/>'
                     f'<axis xyz="0 0 1"/><limit lower="-3" upper="3"/></joint>')
    parts.append("</robot>")
    spheres = {}
    leaf_set = {i for g in pm["env_groups"] for i in g["leaves"]}
    for i, s in enumerate(pm["spheres"]):
        if reference_pairs_only and i not in leaf_set:
            continue          # pRRTC's gate spheres bound leaves; they are not collision geometry
        spheres.setdefault(link[s["frame"]], []).append([*s["c"], s["r"]])
    allowed = []
    if reference_pairs_only:
        sp = pm["spheres"]
        checked = {frozenset((link[sp[a]["frame"]], link[sp[b]["frame"]]))
                   for g in pm["self_groups"] for a, b in g["pairs"]}
        names = list(link.values())
        allowed = [(a, b) for i, a in enumerate(names) for b in names[i + 1:] if frozenset((a, b)) not in checked]
    m = urdf.build_model("".join(parts), spheres, "panda_rt", allowed=allowed)
    src = {}
    for i, s in enumerate(pm["spheres"]):
        if not reference_pairs_only or i in leaf_set:
            src.setdefault(link[s["frame"]], []).append(i)
    doc_order = ["world"] + [link[j["q"]] for j in pm["joints"]]   # the URDF's link order
    idx = [k for lk in doc_order for k in src.get(lk, [])]
    return m, pm, idx


def test_panda_round_trip():
    """Panda's fitted model written out as a URDF and read back gives the
    same sphere kinematics."""
    m, pm, idx = panda_round_trip()
    leaves = [i for g in m["env_groups"] for i in g["leaves"]]
    assert len(leaves) == len(idx) == len(pm["spheres"])
    rng = np.random.default_rng(1)
    for _ in range(10):
        q = rng.uniform(-2.5, 2.5, 7)
        np.testing.assert_allclose(model_centres(m, q)[leaves], model_centres(pm, q)[idx], atol=1e-12)


def test_generated_checker_compiles(tmp_path):
    """codegen turns the URDF model into C tables and a CUDA checker that
    compiles for sm_103a beside the library's own device code."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not shutil.which(nvcc) and not __import__("os").path.exists(nvcc):
        pytest.skip("nvcc not available")
    from pathlib import Path
    from prrtc_gb300.robots import codegen, urdf
    m = urdf.build_model(ARM, SPHERES, "arm")
    (tmp_path / "arm_model.h").write_text(codegen.emit_c_tables(m).replace('#include "model_types.h"', '#include "robots/model_types.h"'))
    (tmp_path / "arm_fkcc.cuh").write_text(codegen.emit_cuda_checker(m))
    csrc = Path(codegen.__file__).resolve().parents[1] / "csrc"
    (tmp_path / "k.cu").write_text(
        '#include "device_common.cuh"\n#include "arm_model.h"\n#include "arm_fkcc.cuh"\n'
        "__global__ void k(const float *q, prrtc::EnvView e, unsigned char *out) {\n"
        "    prrtc::CheckCtx ctx{e, 0.0f, nullptr};\n"
        "    out[threadIdx.x] = prrtc::gen_arm::fkcc(q + 4 * threadIdx.x, ctx) ? 1 : 0;\n"
        "    out[threadIdx.x] &= prrtc::gen_arm::fkcc_validate(q + 4 * threadIdx.x, ctx) ? 1 : 0;\n}\n")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-c", str(tmp_path / "k.cu"),
                        "-o", str(tmp_path / "k.o"), f"-I{csrc}", f"-I{tmp_path}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
