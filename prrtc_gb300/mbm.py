"""MotionBenchMaker problem loader (scene I/O), restating the reference's.

pRRTC's drivers read ``scripts/<robot>_problems.json`` with nlohmann_json and
build an Environment per problem (problem_dict_to_env,
scripts/evaluate_mbm.cpp:13-86):

* spheres -> spheres;
* cylinders -> capsules from centre, Euler XYZ, radius and length
  (factory.hh cylinder::center), except in the ``box`` family, where each
  cylinder becomes a cuboid with half-extents (r, r, r/2)
  (evaluate_mbm.cpp:27-39);
* boxes -> cuboids from centre, Euler XYZ and half-extents (factory.hh cuboid).

Problems whose ``valid`` flag is false are skipped (evaluate_mbm.cpp:131).
No problem data ships with this package; pass the path of a problems file.
"""
from __future__ import annotations

import json
from dataclasses import dataclass

import numpy as np

from .env import Environment, cuboid_row, cylinder_capsule_row


@dataclass
class MbmProblem:
    family: str
    index: int
    env: Environment
    start: np.ndarray
    goals: np.ndarray


def problem_to_env(problem: dict, family: str) -> Environment:
    spheres = [[*o["position"], o["radius"]] for o in problem.get("sphere", [])]
    capsules, cuboids = [], []
    for o in problem.get("cylinder", []):
        r = float(o["radius"])
        if family == "box":
            cuboids.append(cuboid_row(o["position"], (r, r, np.float32(r) / np.float32(2.0)), o["orientation_euler_xyz"]))
        else:
            capsules.append(cylinder_capsule_row(o["position"], o["orientation_euler_xyz"], float(o["length"]), r))
    for o in problem.get("box", []):
        cuboids.append(cuboid_row(o["position"], o["half_extents"], o["orientation_euler_xyz"]))
    return Environment(spheres=np.array(spheres, np.float32).reshape(-1, 4),
                       capsules=np.array(capsules, np.float32).reshape(-1, 8),
                       cuboids=np.array(cuboids, np.float32).reshape(-1, 15))


def load_problems(path) -> list:
    with open(path) as f:
        data = json.load(f)
    out = []
    for family, pset in data["problems"].items():
        for i, p in enumerate(pset):
            if not p.get("valid", False):
                continue
            out.append(MbmProblem(family, i, problem_to_env(p, family), np.asarray(p["start"], np.float32),
                                  np.asarray(p["goals"], np.float32).reshape(len(p["goals"]), -1)))
    return out
