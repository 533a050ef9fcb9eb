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
def test_cli_primal_regression(case, tmp_path, monkeypatch):
    import shutil
    from goal_gb300 import cli
    monkeypatch.chdir(tmp_path)
    c = _cases()[case]
    shutil.copy(os.path.join(ROOT, "tests", "golden", "cube_mesh.npz"), tmp_path / "cube.npz")
    y = tmp_path / "input.yaml"
    y.write_text(reference_style_yaml(case, c, "cube.npz"))
    lines = []
    J = cli.primal(str(y), out=lines.append)
    assert abs(J - c["value"]) < c["tolerance"]
    assert any(l.startswith(" > J(uH) = ") for l in lines)
    assert any("regression" in l for l in lines)


GOAL_INPUTS = os.path.join(ROOT, "tests", "golden", "goal_inputs")
REFERENCE_CASES = ["neohookean_uniaxial_3D", "J2_uniaxial_3D", "J2_traction_3D"]


def _reference_yaml(case):
    return os.path.join(GOAL_INPUTS, "example", "primal", f"{case}.yaml")


@pytest.mark.parametrize("case", REFERENCE_CASES)
def test_reference_input_files_load(case):
    """The reference's own example files, unchanged: the YAML parses with the
    keys the driver accepts, and the mesh it names (cube.smb: the 4-part
    SCOREC mesh cube0.smb .. cube3.smb, joined) is the reference's serial test
    mesh with the same node, side and element sets."""
    import numpy as np
    from goal_gb300 import cli, smb
    _, p = cli._problem(_reference_yaml(case))  # (J2_traction_3D.yaml's list is named "J2 uniaxial 3D")
    assert p["regression"]["value"] == _cases()[case]["value"]
    base = os.path.dirname(_reference_yaml(case))
    dp = p["discretization"]
    assert dp["mesh file"] == "../../test/mesh/cube/cube.smb"
    joined = smb.load(cli._resolve(base, dp["geom file"]), cli._resolve(base, dp["mesh file"]),
                      cli._resolve(base, dp["assoc file"]))
    cube = os.path.join(GOAL_INPUTS, "test", "mesh", "cube")
    serial = smb.load(os.path.join(cube, "cube.dmg"), os.path.join(cube, "cube-serial0.smb"),
                      os.path.join(cube, "cube.txt"))
    assert (joined.num_nodes, joined.num_elems) == (serial.num_nodes, serial.num_elems) == (51, 132)

    def tets(m):
        return sorted(tuple(sorted(map(tuple, m.coords[t]))) for t in m.tets)

    assert tets(joined) == tets(serial)
    for k in serial.node_sets:
        assert sorted(map(tuple, joined.coords[joined.node_sets[k]])) == sorted(map(tuple, serial.coords[serial.node_sets[k]]))
    for k in serial.side_sets:
        assert np.asarray(joined.side_sets[k]).shape == np.asarray(serial.side_sets[k]).shape


@pytest.mark.gpu
@pytest.mark.parametrize("case", REFERENCE_CASES)
def test_cli_primal_on_reference_input_files(case, tmp_path, monkeypatch):
    """GoalPrimal (src/main_primal.cpp:68-90) on the reference's example file
    itself, byte for byte: its mesh, boundary conditions, material, Newton
    settings and regression check (src/goal_regression.cpp:14-23) pass."""
    from goal_gb300 import cli
    monkeypatch.chdir(tmp_path)  # output files land in the working directory, as in goal
    lines = []
    J = cli.primal(_reference_yaml(case), out=lines.append)
    c = _cases()[case]
    assert abs(J - c["value"]) < c["tolerance"]
    assert sum(l.startswith(" > J(uH) = ") for l in lines) == c["num_steps"]
    assert any(l.startswith(" > regression: ") for l in lines)


def _with_output(text, **opts):
    extra = "".join(f"    {k}: {v}\n" for k, v in opts.items())
    return text.replace("  output:\n", "  output:\n" + extra)


@pytest.mark.gpu
def test_cli_output_and_restart(tmp_path, monkeypatch):
    """Three J2 load steps in one run equal two steps, a native restart and
    the third step; every step writes a ParaView dataset."""
    import shutil
    import xml.etree.ElementTree as ET
    from goal_gb300 import cli
    monkeypatch.chdir(tmp_path)
    case = "J2_uniaxial_3D"
    c = dict(_cases()[case])
    shutil.copy(os.path.join(ROOT, "tests", "golden", "cube_mesh.npz"), tmp_path / "cube.npz")
    full = tmp_path / "full.yaml"
    full.write_text(reference_style_yaml(case, c, "cube.npz"))
    J_full = cli.primal(str(full), out=lambda s: None)
    assert abs(J_full - c["value"]) < c["tolerance"]
    pvd = ET.parse(tmp_path / f"out_{case}.pvd").getroot()
    assert len(pvd.find("Collection")) == c["num_steps"]
    vtu = ET.parse(tmp_path / f"out_{case}_0" / f"out_{case}_00.vtu").getroot()
    piece = vtu.find("UnstructuredGrid").find("Piece")
    assert int(piece.get("NumberOfCells")) == 132 and int(piece.get("NumberOfPoints")) == 51
    names = {a.get("Name") for a in piece.iter("DataArray")}
    assert {"u", "p", "sigma", "Fp", "eqps"} <= names

    first = dict(c, num_steps=2, value=0.0, tolerance=1.0)
    y1 = tmp_path / "first.yaml"
    y1.write_text(_with_output(reference_style_yaml(case, first, "cube.npz").replace(
        f"out file: out_{case}", "out file: out_first"), **{"write native": "true"}))
    cli.primal(str(y1), out=lambda s: None)
    assert (tmp_path / "out_first_1" / "restart.npz").exists()
    second = dict(c, num_steps=1)
    y2 = tmp_path / "second.yaml"
    y2.write_text(reference_style_yaml(case, second, "out_first_1/").replace(
        "initial time: 0.0", "initial time: 2.0").replace(f"out file: out_{case}", "out file: out_second"))
    J_restart = cli.primal(str(y2), out=lambda s: None)
    assert J_restart == J_full


@pytest.mark.gpu
def test_cli_nested_adapts_and_the_estimate_predicts_the_change(tmp_path, monkeypatch):
    """GoalNested with two adaptation cycles per load step: the DWR estimate
    z.R printed before each adaptation predicts the change of the QoI that the
    refinement then produces (the nested mesh is the uniform refinement, the
    adapted one a local refinement of it), the mesh grows, and the final QoI
    stays within the reference's tolerance of its regression value (this
    problem's avg disp hardly depends on the mesh)."""
    import shutil
    from goal_gb300 import cli
    monkeypatch.chdir(tmp_path)
    case = "J2_uniaxial_3D"
    c = _cases()[case]
    shutil.copy(os.path.join(ROOT, "tests", "golden", "cube_mesh.npz"), tmp_path / "cube.npz")
    text = reference_style_yaml(case, c, "cube.npz").replace(
        "  output:\n", "  adjoint mode: uniform\n  adaptation:\n    adapt cycles: 2\n    target elems: 1000\n"
                       "    target growth: 2.0\n  output:\n")
    y = tmp_path / "nested.yaml"
    y.write_text(text)
    lines = []
    r = cli.nested(str(y), out=lines.append)
    assert abs(r["J"] - c["value"]) < c["tolerance"]
    assert sum(l.startswith(" > z.R = ") for l in lines) == 2 * c["num_steps"]
    assert sum(l.startswith(" > |J(u)-J(uh)| < ") for l in lines) == 2 * c["num_steps"]
    cyc = r["cycles"]
    assert cyc[-1]["elements"] > 4 * cyc[0]["elements"]
    for k in range(len(cyc) - 1):
        a, b = cyc[k], cyc[k + 1]
        if a["step"] == b["step"] and "eta" in a and abs(a["eta"]) > 1e-13:
            assert abs((b["J"] - a["J"]) - a["eta"]) <= 0.1 * abs(a["eta"]), (a, b)
