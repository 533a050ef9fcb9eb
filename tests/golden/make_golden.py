"""Generates the golden fixtures under tests/golden/ from the reference tree.

Run in a container that has the reference checked out; its root directory is
the one required argument:
    python tests/golden/make_golden.py <reference root>

* cube_mesh.npz   -- the reference's 3D test mesh (test/mesh/cube/cube-serial0.smb
  with cube.dmg and cube.txt), decoded by goal_gb300.smb into coordinates,
  positively oriented tets and the node/side/element sets of cube.txt.
* regression.json -- the regression QoI values the reference's examples assert
  (src/goal_regression.cpp:14-23) for the 3D cases on that mesh, with the
  inputs of each YAML file restated as data.
* goal_inputs/    -- the reference's own input files for those cases, copied
  byte for byte with the directory layout their relative paths expect:
  example/primal/{neohookean_uniaxial_3D,J2_uniaxial_3D,J2_traction_3D}.yaml
  and test/mesh/cube/{cube.dmg, cube.txt, cube0..3.smb (the 4-part mesh the
  YAML files name as cube.smb), cube-serial0.smb}.
"""
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from goal_gb300 import smb  # noqa: E402


def main(ref):
    d = os.path.join(ref, "test", "mesh", "cube")
    m = smb.load(os.path.join(d, "cube.dmg"), os.path.join(d, "cube-serial0.smb"), os.path.join(d, "cube.txt"))
    arrays = dict(coords=m.coords, tets=m.tets, elem_set=m.elem_set)
    for k, v in m.node_sets.items():
        arrays["ns_" + k] = v
    for k, v in m.side_sets.items():
        arrays["ss_" + k] = v
    np.savez(os.path.join(HERE, "cube_mesh.npz"), **arrays)

    base = [[0, "xmin", "0.0"], [1, "ymin", "0.0"], [2, "zmin", "0.0"]]
    cases = {
        "neohookean_uniaxial_3D": dict(
            source="example/primal/neohookean_uniaxial_3D.yaml:1-37",
            model="neohookean", E=1000.0, nu=0.25, K=0.0, Y=0.0, c0=1.0,
            dirichlet=base + [[0, "xmax", "0.01*t"]], traction=[],
            num_steps=3, step_size=1.0, newton_tol=1e-8, newton_max_iters=5,
            functional="avg disp", value=2.541285341193943e-03, tolerance=1.0e-8),
        "J2_uniaxial_3D": dict(
            source="example/primal/J2_uniaxial_3D.yaml:1-39",
            model="J2", E=1000.0, nu=0.25, K=100.0, Y=10.0, c0=1.0,
            dirichlet=base + [[0, "xmax", "0.01*t"]], traction=[],
            num_steps=3, step_size=1.0, newton_tol=1e-8, newton_max_iters=5,
            functional="avg disp", value=1.073955612775838e-03, tolerance=1.0e-8),
        "J2_traction_3D": dict(
            source="example/primal/J2_traction_3D.yaml:1-40",
            model="J2", E=1000.0, nu=0.25, K=100.0, Y=10.0, c0=1.0,
            dirichlet=base, traction=[["ymax", "0.0", "1.0*t", "0.0"]],
            num_steps=3, step_size=1.0, newton_tol=1e-8, newton_max_iters=5,
            functional="avg disp", value=2.512233163668167e-04, tolerance=1.0e-8),
    }
    with open(os.path.join(HERE, "regression.json"), "w") as f:
        json.dump(dict(mesh="cube_mesh.npz", mesh_source="test/mesh/cube/cube-serial0.smb, cube.dmg, cube.txt",
                       cases=cases), f, indent=1)


    inputs = os.path.join(HERE, "goal_inputs")
    for rel in ["example/primal/neohookean_uniaxial_3D.yaml", "example/primal/J2_uniaxial_3D.yaml",
                "example/primal/J2_traction_3D.yaml", "test/mesh/cube/cube.dmg", "test/mesh/cube/cube.txt",
                "test/mesh/cube/cube-serial0.smb"] + [f"test/mesh/cube/cube{k}.smb" for k in range(4)]:
        dst = os.path.join(inputs, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(ref, rel), dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference root>")
    main(sys.argv[1])
