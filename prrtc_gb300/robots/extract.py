"""Derive compact kinematic collision models from pRRTC's generated checkers.

pRRTC's per-robot ``fkcc<Robot>`` (``src/planning/utils.cuh``) is ~1-2 k lines
of straight-line quaternion arithmetic per robot.  This tool does not carry
that code over.  It evaluates it in float64 (``refparse``) and fits, from
those evaluations alone, a much smaller model of the same robot:

* a serial (or tree) chain of joints, each a rotation about (or translation
  along) the local z axis of a frame fixed to its parent body, stored as one
  constant 3x4 transform per joint;
* every collision sphere as (body frame, centre in that frame, radius);
* the checker's decision structure: environment groups (a gating bounding
  sphere and the leaf spheres tested when the gate touches an obstacle) and
  self-collision groups (a gating pair of bounding spheres and the leaf pairs
  tested when the gate overlaps).

The fit uses the product-of-exponentials form: with every joint at zero the
robot is at its home pose; moving one joint alone moves all spheres behind it
rigidly about (or along) that joint's world axis, which a least-squares
rigid-motion fit recovers to float64 round-off.  The fitted model is then
checked against the float64 evaluation of the generated code on random
configurations (``max_err`` in the output).  It is below 3e-7 m for every
robot; the residual is the reference's own: its generated code rounds
constants such as 1/sqrt(2) to 7 digits, so its rotations are orthogonal only
to ~1e-7.

Usage (reads a pRRTC checkout; writes the tables the CUDA code compiles in):

    python -m prrtc_gb300.robots.extract /path/to/pRRTC
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

from . import codegen
from . import refparse as rp

HERE = Path(__file__).resolve().parent
ROBOTS = ("panda", "fetch", "baxter")


def _sphere_keys(prog):
    """Unique spheres (centre operands + radius) in first-use order."""
    keys, index = [], {}
    for t, _ in rp.iter_tests(prog.tests):
        chunks = [t.args] if t.kind == "env" else [t.args[:4], t.args[4:]]
        for c in chunks:
            k = tuple(c)
            if k not in index:
                index[k] = len(keys)
                keys.append(k)
    return keys, index


def _centres(prog, keys, q):
    vals = rp.evaluate(prog, q)
    n = q.shape[0]
    out = np.empty((len(keys), n, 3))
    for i, k in enumerate(keys):
        for a in range(3):
            out[i, :, a] = rp.operand_value(vals, k[a], n)
    return out


def _rigid_fit(p, q):
    """Least-squares R, t with q ~= R p + t (Kabsch)."""
    cp, cq = p.mean(0), q.mean(0)
    h = (p - cp).T @ (q - cq)
    u, _, vt = np.linalg.svd(h)
    d = np.sign(np.linalg.det(vt.T @ u.T))
    r = vt.T @ np.diag([1.0, 1.0, d]) @ u.T
    return r, cq - r @ cp


def _rot_about_z(theta):
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def _frame_from_axis(origin, z, x_hint):
    z = z / np.linalg.norm(z)
    x = x_hint - z * (x_hint @ z)
    if np.linalg.norm(x) < 1e-6:
        x = np.array([0.0, 1.0, 0.0]) - z * z[1]
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    h = np.eye(4)
    h[:3, 0], h[:3, 1], h[:3, 2], h[:3, 3] = x, y, z, origin
    return h


def _snap(m, tol=1e-6):
    """Remove the reference's ~1e-7 rounding noise: entries within ``tol`` of
    0 or +-1 become exact, and other entries within 5e-8 of a multiple of 1e-6
    are rounded to it (URDF dimensions are given to <= 6 decimals)."""
    m = np.array(m, dtype=np.float64)
    for v in (0.0, 1.0, -1.0):
        m[np.abs(m - v) < tol] = v
    r = np.round(m, 6)
    near = np.abs(m - r) < 5e-8
    m[near] = r[near]
    return m


def fit_model(prog, rng_seed=0):
    keys, index = _sphere_keys(prog)
    dep = rp.dependencies(prog)
    D = prog.dof
    sph_dep = []
    for k in keys:
        s = frozenset()
        for a in k[:3]:
            if isinstance(a, str):
                s |= dep[a]
        sph_dep.append(s)

    # bodies: distinct dependency sets.  A joint's chain position is the number
    # of joints in front of it; the generated code is a tree of serial chains,
    # so every body's set is {its joint} plus that joint's ancestors.
    body_sets = sorted(set(sph_dep), key=lambda s: (len(s), sorted(s)))
    joint_parent = {}
    joint_body = {}
    for s in body_sets:
        if not s:
            continue
        # the body's own joint is the one not present in any strict subset body
        subs = [b for b in body_sets if b < s]
        parent_set = max(subs, key=len) if subs else frozenset()
        own = s - parent_set
        if len(own) != 1:
            raise ValueError(f"{prog.robot}: body {sorted(s)} adds {len(own)} joints; a sphere-free link in a chain is not supported")
        j = next(iter(own))
        joint_body[j] = s
        parent_joints = [jj for jj, bs in joint_body.items() if bs == parent_set]
        joint_parent[j] = parent_joints[0] if parent_joints else -1
    if sorted(joint_body) != list(range(D)):
        raise ValueError(f"{prog.robot}: joints without spheres: {set(range(D)) - set(joint_body)}")

    home = _centres(prog, keys, np.zeros((1, D)))[:, 0, :]

    # world screw of each joint at home
    screws = {}
    for j in range(D):
        moving = [i for i, s in enumerate(sph_dep) if j in s]
        pts0 = home[moving]
        kinds = []
        for theta in (0.9, -0.6):
            qq = np.zeros((1, D))
            qq[0, j] = theta
            pts = _centres(prog, keys, qq)[moving, 0, :]
            disp = pts - pts0
            if np.ptp(disp, axis=0).max() < 1e-12:          # pure translation
                v = disp.mean(0) / theta
                kinds.append(("prismatic", v, None))
                continue
            r, t = _rigid_fit(pts0, pts)
            ang = np.arccos(np.clip((np.trace(r) - 1) / 2, -1, 1))
            w = np.array([r[2, 1] - r[1, 2], r[0, 2] - r[2, 0], r[1, 0] - r[0, 1]])
            w /= np.linalg.norm(w)
            if abs(ang - abs(theta)) > 1e-5:
                raise ValueError(f"{prog.robot}: joint {j} is not a unit-rate revolute ({ang} vs {theta})")
            if theta < 0:
                w = -w
            # point on the axis: least-squares solution of (I - R) a = t
            a = np.linalg.lstsq(np.eye(3) - r, t, rcond=None)[0]
            kinds.append(("revolute", w, a))
        k0, k1 = kinds
        if k0[0] != k1[0] or np.abs(k0[1] - k1[1]).max() > 1e-5:
            raise ValueError(f"{prog.robot}: joint {j} screw is not consistent")
        if k0[0] == "prismatic" and abs(np.linalg.norm(k0[1]) - 1) > 1e-5:
            raise ValueError(f"{prog.robot}: prismatic joint {j} is not unit rate")
        screws[j] = k0

    # local frames: joint j's frame has z along its axis
    order = sorted(range(D), key=lambda j: len(joint_body[j]))
    H = {-1: np.eye(4)}
    for j in order:
        kind, w, a = screws[j]
        ph = H[joint_parent[j]]
        if kind == "revolute":
            # origin: point of the axis closest to the parent frame origin
            o = a + w * ((ph[:3, 3] - a) @ w)
        else:
            o = ph[:3, 3].copy()
        H[j] = _frame_from_axis(o, w, ph[:3, 0])

    joints = []
    for j in order:
        kind, _, _ = screws[j]
        p = joint_parent[j]
        F = np.linalg.inv(H[p]) @ H[j]
        F[:3, :3] = _snap(F[:3, :3])
        F[:3, 3] = _snap(F[:3, 3], 1e-7)
        joints.append({"q": j, "parent": p, "type": kind, "F": F[:3, :].tolist()})
    # recompute H from the snapped transforms so the sphere positions are
    # expressed consistently with what the kernels evaluate
    Hs = {-1: np.eye(4)}
    for jt in joints:
        F = np.eye(4)
        F[:3, :] = np.array(jt["F"])
        Hs[jt["q"]] = Hs[jt["parent"]] @ F

    body_joint = {frozenset(): -1}
    for j, s in joint_body.items():
        body_joint[s] = j
    spheres = []
    for i, k in enumerate(keys):
        f = body_joint[sph_dep[i]]
        pl = np.linalg.inv(Hs[f]) @ np.append(home[i], 1.0)
        spheres.append({"frame": f, "c": _snap(pl[:3], 1e-7).tolist(), "r": float(k[3])})

    env_groups, self_groups, schedule = [], [], []
    for t in prog.tests:
        schedule.append([t.kind, len(env_groups) if t.kind == "env" else len(self_groups)])
        if t.kind == "env":
            if t.returns and not t.children:
                env_groups.append({"gate": -1, "leaves": [index[tuple(t.args)]], "label": t.label})
            else:
                if t.returns or any(c.children or c.kind != "env" or not c.returns for c in t.children):
                    raise ValueError("unsupported env block shape")
                env_groups.append({"gate": index[tuple(t.args)],
                                   "leaves": [index[tuple(c.args)] for c in t.children], "label": t.label})
        else:
            if t.returns and not t.children:
                self_groups.append({"gate": None,
                                    "pairs": [[index[tuple(t.args[:4])], index[tuple(t.args[4:])]]], "label": t.label})
            else:
                if t.returns or any(c.children or c.kind != "self" or not c.returns for c in t.children):
                    raise ValueError("unsupported self block shape")
                self_groups.append({"gate": [index[tuple(t.args[:4])], index[tuple(t.args[4:])]],
                                    "pairs": [[index[tuple(c.args[:4])], index[tuple(c.args[4:])]] for c in t.children],
                                    "label": t.label})
    model = {"robot": prog.robot, "dof": D, "joints": joints, "spheres": spheres,
             "env_groups": env_groups, "self_groups": self_groups, "schedule": schedule}

    rng = np.random.default_rng(rng_seed)
    q = rng.uniform(-np.pi, np.pi, size=(2000, D))
    ref = _centres(prog, keys, q)
    got = model_sphere_centres(model, q)
    model["max_err"] = float(np.abs(ref - got).max())
    return model


def model_frames(model, q):
    """World 4x4 frame of every joint (index = config index) for q (N, D)."""
    q = np.asarray(q, dtype=np.float64)
    n = q.shape[0]
    T = {-1: np.broadcast_to(np.eye(4), (n, 4, 4))}
    for jt in model["joints"]:
        F = np.eye(4)
        F[:3, :] = np.array(jt["F"])
        th = q[:, jt["q"]]
        M = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
        if jt["type"] == "revolute":
            c, s = np.cos(th), np.sin(th)
            M[:, 0, 0], M[:, 0, 1], M[:, 1, 0], M[:, 1, 1] = c, -s, s, c
        else:
            M[:, 2, 3] = th
        T[jt["q"]] = T[jt["parent"]] @ F @ M
    return T


def model_sphere_centres(model, q, only=None):
    """(S, N, 3) float64 world centres of the model spheres (all, or the
    indices in `only`, in that order)."""
    q = np.asarray(q, dtype=np.float64)
    idx = range(len(model["spheres"])) if only is None else list(only)
    sph = [model["spheres"][i] for i in idx]
    if only is not None:
        needed = {s["frame"] for s in sph}
        sub = dict(model)
        keep = set()
        parent = {jt["q"]: jt["parent"] for jt in model["joints"]}
        for f in needed:
            while f >= 0 and f not in keep:
                keep.add(f)
                f = parent[f]
        sub["joints"] = [jt for jt in model["joints"] if jt["q"] in keep]
        T = model_frames(sub, q)
    else:
        T = model_frames(model, q)
    out = np.empty((len(sph), q.shape[0], 3))
    for i, s in enumerate(sph):
        Tf = T[s["frame"]]
        out[i] = Tf[:, :3, :3] @ np.array(s["c"]) + Tf[:, :3, 3]
    return out


def sphere_robot_model():
    """pRRTC's toy 3-DoF point robot (``Robots.hh:190-237``, ``utils.cuh:330-334``):
    a radius-1 sphere translated by (q0, q1, q2)."""
    I = np.eye(4)
    joints = []
    # each frame's z is its parent's x: frames 0, 1, 2 slide along world x, y, z
    cyc = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]])
    for j in range(3):
        F = I.copy()
        F[:3, :3] = cyc
        joints.append({"q": j, "parent": j - 1, "type": "prismatic", "F": F[:3, :].tolist()})
    model = {"robot": "sphere", "dof": 3, "joints": joints,
             "spheres": [{"frame": 2, "c": [0.0, 0.0, 0.0], "r": 1.0}],
             "env_groups": [{"gate": -1, "leaves": [0], "label": "sphere"}], "self_groups": [],
             "schedule": [["env", 0]]}
    q = np.random.default_rng(0).uniform(-5, 5, size=(100, 3))
    model["max_err"] = float(np.abs(model_sphere_centres(model, q)[0] - q).max())
    return model


def main(argv):
    if len(argv) != 2:
        print(__doc__)
        return 2
    ref = Path(argv[1])
    models = {}
    for r in ROBOTS:
        prog = rp.load_program(ref, r)
        models[r] = fit_model(prog)
    models["sphere"] = sphere_robot_model()
    for r, m in models.items():
        (HERE / f"{r}.json").write_text(json.dumps(m, indent=1) + "\n")
        print(f"{r}: dof={m['dof']} spheres={len(m['spheres'])} env_groups={len(m['env_groups'])} "
              f"self_groups={len(m['self_groups'])} max_err={m['max_err']:.2e}")
    codegen.write_all()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
