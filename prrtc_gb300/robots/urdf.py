"""Robot-model compiler front end for new robots: a URDF plus collision spheres
-> the JSON model that ``codegen.py`` compiles into C tables and a CUDA
checker.

pRRTC's own robots come from its generated checkers (``extract.py`` fits
them).  A new robot needs only its kinematics and a sphere model:

* ``urdf``: revolute, continuous, prismatic and fixed joints, each with an
  ``origin`` (xyz, rpy: R = Rz(yaw) Ry(pitch) Rx(roll)) and an ``axis``;
  joint ``limit`` lower/upper give the sampler's joint box;
* ``spheres``: ``{link name: [[x, y, z, r], ...]}`` in that link's frame;
* ``allowed``: extra link pairs never checked against each other (links
  joined by a joint are never checked, as is usual for sphere models).

Model conventions (``model_types.h``): every movable joint is a frame that
rotates about (or slides along) its local z.  A URDF joint with axis a
becomes F = X_parent * O * A, where O is the joint's origin, X_parent the
fixed transform from the parent link's body frame, and A a rotation taking z
to a; the child link's frame is then J * Rz(q) * A^T.  Fixed joints fold into
the links' transforms, and every sphere is stored in the frame of the movable
joint it rides on.

The checker hierarchy is generated: one environment group per link with
spheres (gate: a bounding sphere of the link's spheres), and one self group
per pair of checked links (gate: the two bounding spheres), environment
groups first, in URDF order.

    python -m prrtc_gb300.robots.urdf robot.urdf spheres.json name   # writes robots/<name>.json
"""
from __future__ import annotations

import json
import math
import sys
import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def rpy_matrix(r: float, p: float, y: float) -> np.ndarray:
    """URDF orientation: R = Rz(y) Ry(p) Rx(r)."""
    cr, sr, cp, sp, cy, sy = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(y), math.sin(y)
    Rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    Ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    Rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def homogeneous(R: np.ndarray, t) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def align_z(a) -> np.ndarray:
    """A rotation whose third column is the unit vector a (A z = a)."""
    a = np.asarray(a, float)
    a = a / np.linalg.norm(a)
    if abs(a[2] - 1.0) < 1e-12:
        return np.eye(3)
    if abs(a[2] + 1.0) < 1e-12:
        return np.diag([1.0, -1.0, -1.0])   # rotation by pi about x
    helper = np.array([1.0, 0.0, 0.0]) if abs(a[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    x = helper - a * (helper @ a)
    x /= np.linalg.norm(x)
    y = np.cross(a, x)
    return np.column_stack([x, y, a])


def parse_urdf(text: str) -> tuple[list, list]:
    """(links, joints) of a URDF document; joints in document order."""
    root = ET.fromstring(text)
    links = [l.get("name") for l in root.findall("link")]
    joints = []
    for j in root.findall("joint"):
        o = j.find("origin")
        xyz = [float(v) for v in (o.get("xyz", "0 0 0") if o is not None else "0 0 0").split()]
        rpy = [float(v) for v in (o.get("rpy", "0 0 0") if o is not None else "0 0 0").split()]
        ax = j.find("axis")
        axis = [float(v) for v in (ax.get("xyz") if ax is not None else "1 0 0").split()]
        lim = j.find("limit")
        lower = float(lim.get("lower", "0")) if lim is not None else 0.0
        upper = float(lim.get("upper", "0")) if lim is not None else 0.0
        jtype = j.get("type")
        if jtype == "continuous":
            jtype, lower, upper = "revolute", -math.pi, math.pi
        joints.append({"name": j.get("name"), "type": jtype, "parent": j.find("parent").get("link"),
                       "child": j.find("child").get("link"), "xyz": xyz, "rpy": rpy, "axis": axis,
                       "lower": lower, "upper": upper})
    return links, joints


def build_model(urdf_text: str, spheres: dict, name: str, allowed=()) -> dict:
    """The codegen model of a URDF and its per-link spheres."""
    links, joints = parse_urdf(urdf_text)
    children = {j["child"] for j in joints}
    roots = [l for l in links if l not in children]
    if len(roots) != 1:
        raise ValueError(f"expected one root link, found {roots}")
    body = {roots[0]: -1}              # link -> config index of its movable frame (-1 world)
    X = {roots[0]: np.eye(4)}          # link -> transform from that frame to the link
    model_joints, limits = [], []
    pending = list(joints)
    while pending:                     # parents before children, document order otherwise
        progressed = False
        for j in list(pending):
            if j["parent"] not in body:
                continue
            pending.remove(j)
            progressed = True
            O = homogeneous(rpy_matrix(*j["rpy"]), j["xyz"])
            XP = X[j["parent"]]
            if j["type"] == "fixed":
                body[j["child"]] = body[j["parent"]]
                X[j["child"]] = XP @ O
                continue
            if j["type"] not in ("revolute", "prismatic"):
                raise ValueError(f"joint {j['name']}: unsupported type {j['type']}")
            A = align_z(j["axis"])
            F = XP @ O @ homogeneous(A, [0.0, 0.0, 0.0])
            q = len(model_joints)
            model_joints.append({"q": q, "parent": body[j["parent"]], "type": j["type"],
                                 "F": [[float(v) for v in F[i]] for i in range(3)], "name": j["name"]})
            limits.append((j["lower"], j["upper"]))
            body[j["child"]] = q
            X[j["child"]] = homogeneous(A.T, [0.0, 0.0, 0.0])
        if not progressed:
            raise ValueError("joints do not form a tree")

    sph, link_leaves, link_gate = [], {}, {}
    for link in links:
        rows = spheres.get(link, [])
        if not rows:
            continue
        idx = []
        for x, y, z, r in rows:
            c = X[link] @ np.array([x, y, z, 1.0])
            idx.append(len(sph))
            sph.append({"frame": body[link], "c": [float(v) for v in c[:3]], "r": float(r)})
        link_leaves[link] = idx
        if len(idx) > 1:               # bounding sphere of the link's spheres as its gate
            cs = np.array([sph[i]["c"] for i in idx])
            rs = np.array([sph[i]["r"] for i in idx])
            ctr = (cs.min(0) + cs.max(0)) / 2
            rad = float(np.max(np.linalg.norm(cs - ctr, axis=1) + rs))
            link_gate[link] = len(sph)
            sph.append({"frame": body[link], "c": [float(v) for v in ctr], "r": rad})
        else:
            link_gate[link] = idx[0]

    adjacent = {frozenset((j["parent"], j["child"])) for j in joints}
    adjacent |= {frozenset(p) for p in allowed}
    env_groups, self_groups = [], []
    for link, idx in link_leaves.items():
        env_groups.append({"gate": link_gate[link] if len(idx) > 1 else -1, "leaves": idx, "label": link})
    names = list(link_leaves)
    for a in range(len(names)):
        for b in range(a + 1, len(names)):
            la, lb = names[a], names[b]
            if frozenset((la, lb)) in adjacent or body[la] == body[lb]:
                continue               # joined links, or one rigid body
            pairs = [[i, k] for i in link_leaves[la] for k in link_leaves[lb]]
            self_groups.append({"gate": [link_gate[la], link_gate[lb]], "pairs": pairs, "label": f"{la} vs. {lb}"})
    schedule = [["env", i] for i in range(len(env_groups))] + [["self", i] for i in range(len(self_groups))]
    return {"robot": name, "dof": len(model_joints), "joints": model_joints, "spheres": sph,
            "env_groups": env_groups, "self_groups": self_groups, "schedule": schedule, "max_err": 0.0,
            "limits": {"lower": [l for l, _ in limits], "upper": [u for _, u in limits]}}


def urdf_sphere_centres(urdf_text: str, spheres: dict, q) -> dict:
    """World sphere centres straight from URDF semantics (Rodrigues rotation
    about each joint's axis): an independent check of build_model."""
    links, joints = parse_urdf(urdf_text)
    children = {j["child"] for j in joints}
    root = [l for l in links if l not in children][0]
    W = {root: np.eye(4)}
    qi = 0
    pending = list(joints)
    while pending:
        for j in list(pending):
            if j["parent"] not in W:
                continue
            pending.remove(j)
            T = W[j["parent"]] @ homogeneous(rpy_matrix(*j["rpy"]), j["xyz"])
            if j["type"] != "fixed":
                a = np.asarray(j["axis"], float)
                a /= np.linalg.norm(a)
                if j["type"] == "prismatic":
                    M = homogeneous(np.eye(3), a * q[qi])
                else:
                    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
                    th = q[qi]
                    M = homogeneous(np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * K @ K, [0, 0, 0])
                T = T @ M
                qi += 1
            W[j["child"]] = T
    return {link: [(W[link] @ np.array([x, y, z, 1.0]))[:3] for x, y, z, _ in rows] for link, rows in spheres.items()}


def main(argv):
    urdf_path, spheres_path, name = argv[1], argv[2], argv[3]
    m = build_model(Path(urdf_path).read_text(), json.loads(Path(spheres_path).read_text()), name)
    (HERE / f"{name}.json").write_text(json.dumps(m, indent=1) + "\n")
    print(f"{name}: {m['dof']} joints, {len(m['spheres'])} spheres, {len(m['env_groups'])} environment groups, "
          f"{len(m['self_groups'])} self groups", file=sys.stderr)


if __name__ == "__main__":
    main(sys.argv)
