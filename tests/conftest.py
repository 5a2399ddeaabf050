import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def _reference() -> Path:
    """The pRRTC checkout: $PRRTC_REFERENCE, else the one the oracle's
    reference builds were made from (recorded by the build), else none."""
    env = os.environ.get("PRRTC_REFERENCE")
    if env:
        return Path(env)
    rec = ROOT / "oracle" / "_ref" / "REFERENCE"
    return Path(rec.read_text().strip()) if rec.exists() else ROOT / "oracle" / "_ref" / "no-reference"


REFERENCE = _reference()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(p.stem.replace("checker_", "") for p in GOLDEN.glob("checker_*.npz"))


def load_golden(case: str):
    from prrtc_gb300.env import Environment
    z = np.load(GOLDEN / f"checker_{case}.npz")
    env = Environment(spheres=z["env_spheres"], capsules=z["env_capsules"], z_aligned_capsules=z["env_z_capsules"],
                      cuboids=z["env_cuboids"], z_aligned_cuboids=z["env_z_cuboids"])
    return env, {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle():
    from pyoracle import OracleLib, build
    build()
    return OracleLib()


@pytest.fixture(scope="session")
def ctx():
    import prrtc_gb300.build as b
    b.build()
    from prrtc_gb300 import Context
    c = Context(0)
    yield c
    c.close()
