import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def cube_kat():
    import json
    from goal_gb300.mesh import load_npz
    gdir = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(gdir, "regression.json")) as f:
        reg = json.load(f)
    mesh = load_npz(os.path.join(gdir, reg["mesh"]), ["cube"])
    return mesh, reg["cases"]
