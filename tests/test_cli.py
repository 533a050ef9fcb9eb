"""The YAML input driver: goal's input-file layout parsed by the package's
YAML-subset reader (CPU), and run end to end on the GPU with the regression
check of the reference's example files."""
import json
import os

import pytest

from goal_gb300 import yaml_lite

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_style_yaml(case, c, mesh_file):
    dbc = "\n".join(f"    bc {i + 1}: [{b[0]}, {b[1]}, {b[2]}]" for i, b in enumerate(c["dirichlet"]))
    tbc = "\n".join(f"    bc {i + 1}: [{', '.join(t)}]" for i, t in enumerate(c["traction"]))
    mat = f"        E: {c['E']}\n        nu: {c['nu']}\n        c0: {c['c0']}\n"
    if c["model"] == "J2":
        mat += f"        K: {c['K']}\n        Y: {c['Y']}\n"
    return f"""{case}:
  num steps: {c['num_steps']}
  step size: {c['step_size']}
  initial time: 0.0 
  discretization:
    geom file: 'unused.dmg'
    mesh file: '{mesh_file}'
    assoc file: 'unused.txt'
  dirichlet bcs:
{dbc}
""" + (f"""  traction bcs:
{tbc}
""" if tbc else "") + f"""  mechanics:
    model: {c['model']}
    materials:
      cube:
{mat}  primal linear algebra:
    krylov size: 100
    max iters: 100
    tolerance: 1.0e-10
    multigrid:
      verbosity: none   # comment
      number of equations: 4
    nonlinear tolerance: {c['newton_tol']}
    nonlinear max iters: {c['newton_max_iters']}
  functional:
    type: {c['functional']}
  output:
    out file: out_{case}
  regression:
    value: {c['value']!r}
    tolerance: {c['tolerance']}
"""


def _cases():
    with open(os.path.join(ROOT, "tests", "golden", "regression.json")) as f:
        return json.load(f)["cases"]


def test_yaml_lite_parses_reference_layout():
    c = _cases()["J2_traction_3D"]
    doc = yaml_lite.loads(reference_style_yaml("J2 traction 3D", c, "cube.npz"))
    p = doc["J2 traction 3D"]
    assert p["num steps"] == 3 and p["step size"] == 1.0
    assert p["dirichlet bcs"]["bc 2"] == [1, "ymin", 0.0]
    assert p["traction bcs"]["bc 1"] == ["ymax", 0.0, "1.0*t", 0.0]
    assert p["mechanics"]["materials"]["cube"]["Y"] == 10.0
    assert p["primal linear algebra"]["multigrid"]["verbosity"] == "none"
    assert p["regression"]["value"] == c["value"]
    assert p["discretization"]["mesh file"] == "cube.npz"


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["neohookean_uniaxial_3D", "J2_traction_3D"])
def test_cli_primal_regression(case, tmp_path):
    import shutil
    from goal_gb300 import cli
    c = _cases()[case]
    shutil.copy(os.path.join(ROOT, "tests", "golden", "cube_mesh.npz"), tmp_path / "cube.npz")
    y = tmp_path / "input.yaml"
    y.write_text(reference_style_yaml(case, c, "cube.npz"))
    lines = []
    J = cli.primal(str(y), out=lines.append)
    assert abs(J - c["value"]) < c["tolerance"]
    assert any(l.startswith(" > J(uH) = ") for l in lines)
    assert any("regression" in l for l in lines)
