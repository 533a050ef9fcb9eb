"""goal::Output (src/goal_output.cpp:24-110): ParaView output and native
restart files of a primal run.

* ``<out file>.pvd`` is the collection; every write adds a dataset at time
  t + 1e-4 * cycle (:104-108). The dataset is ``<out file>_<i>/<out file>_<i>.pvtu``
  with one piece ``<out file>_<i>/<out file>_<i>0.vtu`` (one part, as the
  reference's single-rank runs).
* Point data: ``u`` (3 components) and ``p``; cell data: the states ``sigma``,
  ``Fp``, ``eqps`` (J2), their ``_old`` copies, and any extra cell fields the
  caller passes (e.g. error indicators).
* ``write native`` (:88-94) writes ``<out file>_<i>/restart.npz`` instead of an
  SMB file: mesh, node/side sets, the nodal solution and all states. A run
  whose ``mesh file`` names such a directory continues from it
  (``load_restart``).
* ``interval`` and ``turn off`` as in the reference; the interval counter is
  per Output object (the reference keeps it in a function-static variable).
"""
from __future__ import annotations

import base64
import os
import struct

import numpy as np

from . import api
from .mesh import Mesh

VTK_TETRA = 10


def _b64(arr: np.ndarray) -> str:
    raw = np.ascontiguousarray(arr).tobytes()
    return base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode("ascii")


def _data_array(name: str, arr: np.ndarray, ncomp: int) -> str:
    kind = {np.dtype(np.float64): "Float64", np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64",
            np.dtype(np.uint8): "UInt8"}[arr.dtype]
    return (f'        <DataArray type="{kind}" Name="{name}" NumberOfComponents="{ncomp}" format="binary">\n'
            f"          {_b64(arr)}\n        </DataArray>\n")


def write_vtu(path: str, coords: np.ndarray, tets: np.ndarray, point_data: dict, cell_data: dict) -> None:
    """One unstructured-grid piece (VTK XML, base64 binary with 64-bit headers)."""
    N, E = len(coords), len(tets)
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
           "  <UnstructuredGrid>\n", f'    <Piece NumberOfPoints="{N}" NumberOfCells="{E}">\n',
           "      <Points>\n", _data_array("coordinates", np.asarray(coords, np.float64), 3), "      </Points>\n",
           "      <Cells>\n",
           _data_array("connectivity", np.asarray(tets, np.int64).ravel(), 1),
           _data_array("offsets", 4 * np.arange(1, E + 1, dtype=np.int64), 1),
           _data_array("types", np.full(E, VTK_TETRA, np.uint8), 1), "      </Cells>\n", "      <PointData>\n"]
    for name, (arr, nc) in point_data.items():
        out.append(_data_array(name, np.asarray(arr, np.float64).ravel(), nc))
    out.append("      </PointData>\n      <CellData>\n")
    for name, (arr, nc) in cell_data.items():
        out.append(_data_array(name, np.asarray(arr, np.float64).ravel(), nc))
    out.append("      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as f:
        f.write("".join(out))


def write_pvtu(path: str, piece: str, point_data: dict, cell_data: dict) -> None:
    lines = ['<?xml version="1.0"?>\n',
             '<VTKFile type="PUnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n',
             '  <PUnstructuredGrid GhostLevel="0">\n',
             '    <PPoints><PDataArray type="Float64" Name="coordinates" NumberOfComponents="3"/></PPoints>\n',
             "    <PPointData>\n"]
    for name, (_, nc) in point_data.items():
        lines.append(f'      <PDataArray type="Float64" Name="{name}" NumberOfComponents="{nc}"/>\n')
    lines.append("    </PPointData>\n    <PCellData>\n")
    for name, (_, nc) in cell_data.items():
        lines.append(f'      <PDataArray type="Float64" Name="{name}" NumberOfComponents="{nc}"/>\n')
    lines.append(f'    </PCellData>\n    <Piece Source="{piece}"/>\n  </PUnstructuredGrid>\n</VTKFile>\n')
    with open(path, "w") as f:
        f.write("".join(lines))


STATE_FIELDS = (("sigma", api.SIGMA, 9), ("Fp", api.FP, 9), ("Fp_old", api.FP_OLD, 9), ("eqps", api.EQPS, 1),
                ("eqps_old", api.EQPS_OLD, 1))


def _states(mech) -> dict:
    names = STATE_FIELDS if mech.model == api.J2 else STATE_FIELDS[:1]
    return {n: (mech.get_state(w), nc) for n, w, nc in names}


class Output:
    def __init__(self, params: dict, mesh: Mesh, mech, base_dir: str = "."):
        self.name = str(params.get("out file", ""))
        self.interval = int(params.get("interval", 1)) or 1
        self.turn_off = bool(params.get("turn off", False))
        self.write_native = bool(params.get("write native", False))
        self.mesh, self.mech = mesh, mech
        self.root = os.path.join(base_dir, self.name) if self.name else ""
        self.index = 0
        self.calls = 0
        self.datasets = []
        if not self.turn_off and self.name:
            self._write_pvd()

    def _write_pvd(self):
        with open(self.root + ".pvd", "w") as f:
            f.write('<VTKFile type="Collection" version="0.1">\n  <Collection>\n')
            for t, vtu in self.datasets:
                f.write(f'    <DataSet timestep="{t}" group="" part="0" file="{vtu}/{vtu}.pvtu"/>\n')
            f.write("  </Collection>\n</VTKFile>\n")

    def write(self, t: float, cycle: int = 0, cell_fields: dict | None = None) -> None:
        if self.turn_off or not self.name:
            return
        c = self.calls
        self.calls += 1
        if c % self.interval:
            return
        vtu = f"{os.path.basename(self.name)}_{self.index}"
        folder = f"{self.root}_{self.index}"
        os.makedirs(folder, exist_ok=True)
        U = self.mech.get_solution().reshape(-1, 4)
        states = _states(self.mech)
        if self.write_native:
            save_restart(os.path.join(folder, "restart.npz"), self.mesh, U, states)
        point = {"u": (U[:, :3], 3), "p": (U[:, 3], 1)}
        cell = dict(states)
        for k, v in (cell_fields or {}).items():
            cell[k] = (np.asarray(v), 1)
        write_vtu(os.path.join(folder, vtu + "0.vtu"), self.mesh.coords, self.mesh.tets, point, cell)
        write_pvtu(os.path.join(folder, vtu + ".pvtu"), vtu + "0.vtu", point, cell)
        self.datasets.append((t + 1.0e-4 * cycle, vtu))
        self._write_pvd()
        self.index += 1


def save_restart(path: str, mesh: Mesh, U: np.ndarray, states: dict) -> None:
    arrays = {"coords": mesh.coords, "tets": mesh.tets, "elem_set": mesh.elem_set,
              "elem_set_names": np.array(mesh.elem_set_names), "U": U}
    for k, v in mesh.node_sets.items():
        arrays[f"ns:{k}"] = v
    for k, v in mesh.side_sets.items():
        arrays[f"ss:{k}"] = v
    for k, (v, _) in states.items():
        arrays[f"state:{k}"] = v
    np.savez(path, **arrays)


def is_restart(path: str) -> bool:
    return os.path.isdir(path) and os.path.exists(os.path.join(path, "restart.npz"))


def load_restart(path: str):
    """Mesh, nodal solution (N x 4) and states of a native restart directory."""
    z = np.load(os.path.join(path, "restart.npz"))
    mesh = Mesh(coords=z["coords"], tets=z["tets"], elem_set=z["elem_set"],
                elem_set_names=[str(s) for s in z["elem_set_names"]],
                node_sets={k[3:]: z[k] for k in z.files if k.startswith("ns:")},
                side_sets={k[3:]: z[k] for k in z.files if k.startswith("ss:")})
    states = {k[6:]: z[k] for k in z.files if k.startswith("state:")}
    return mesh, z["U"], states


def apply_restart(mech, U: np.ndarray, states: dict) -> None:
    """Continues a run from a restart written after a converged step: the
    solution and the states as written, then States::update (the step's
    states become the old ones, src/goal_states.cpp:130-141), as after that
    step in an uninterrupted run."""
    mech.set_solution(np.ascontiguousarray(U).ravel())
    ids = {n: w for n, w, _ in STATE_FIELDS}
    for k, v in states.items():
        mech.set_state(ids[k], v)
    if mech.model == api.J2:
        mech.update_states()
