"""Robot models: generated code is current, and the fitted models reproduce
the reference's float64 forward kinematics (CPU)."""
import numpy as np
import pytest

from conftest import REFERENCE, golden_cases, load_golden


def test_generated_files_are_current():
    from prrtc_gb300.robots import codegen
    assert codegen.check_up_to_date() == []


def test_single_configuration_checker_forms():
    """The stand-alone checker's form per robot, as measured on the GB300:
    Panda's fkcc_validate is its own straight-line code; Fetch's and
    Baxter's delegate to the table-form walk (fkcc); the sphere robot has
    no table form at all, so both of its entry points are straight-line."""
    from prrtc_gb300.robots import codegen
    head = "bool fkcc_validate(const float *__restrict__ q, Ctx &ctx)\n{\n"
    for robot, delegates, table in (("sphere", True, False), ("panda", False, True), ("fetch", True, True),
                                    ("baxter", True, True)):
        text = (codegen.CSRC / f"{robot}_fkcc.cuh").read_text()
        body = text[text.index(head) + len(head):]
        assert body.startswith("    return fkcc(q, ctx);\n}") == delegates, robot
        assert ("run_schedule(" in text) == table, robot


@pytest.mark.parametrize("case", golden_cases())
def test_model_fk_matches_reference_fp64(case, oracle):
    """Oracle float64 FK of the fitted model vs the reference's generated FK
    evaluated in float64 (fixture): every sphere centre within 1e-6 m."""
    robot = case.split("_")[0]
    env, z = load_golden(case)
    got = oracle.fk_spheres(robot, z["fk_q"].astype(np.float64))[..., :3]
    ref = z["fk_centres"]
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() < 1e-6


@pytest.mark.skipif(not (REFERENCE / "src/planning/utils.cuh").exists(), reason="reference checkout absent")
@pytest.mark.parametrize("robot", ["panda", "fetch", "baxter"])
def test_model_fit_live(robot):
    from prrtc_gb300.robots import extract, refparse
    from prrtc_gb300.scenes import load_model
    prog = refparse.load_program(REFERENCE, robot)
    m = load_model(robot)
    q = np.random.default_rng(7).uniform(-3, 3, (500, prog.dof))
    keys, _ = extract._sphere_keys(prog)
    ref = extract._centres(prog, keys, q)
    got = extract.model_sphere_centres(m, q)
    assert np.abs(ref - got).max() < 1e-6
    # the decision structure counts of the reference (utils.cuh)
    n_leaf = sum(len(g["leaves"]) for g in m["env_groups"])
    n_pair = sum(len(g["pairs"]) for g in m["self_groups"])
    expect = {"panda": (58, 690), "fetch": (111, 2586), "baxter": (75, 1925)}[robot]
    assert (n_leaf, n_pair) == expect
