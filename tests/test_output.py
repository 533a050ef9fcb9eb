"""ParaView files and native restart files of goal_gb300.output
(src/goal_output.cpp), on the CPU: the XML parses, every binary array decodes
to the values written, and a restart directory round-trips the mesh, the sets,
the solution and the states."""
import base64
import struct
import xml.etree.ElementTree as ET

import numpy as np

from goal_gb300 import output
from goal_gb300.mesh import kuhn_cube


def _decode(text, dtype):
    raw = base64.b64decode(text.strip())
    (n,) = struct.unpack("<Q", raw[:8])
    assert n == len(raw) - 8
    return np.frombuffer(raw[8:], dtype=dtype)


def test_vtu_arrays_decode(tmp_path):
    mesh = kuhn_cube(2)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((mesh.num_nodes, 3))
    p = rng.standard_normal(mesh.num_nodes)
    sig = rng.standard_normal((mesh.num_elems, 9))
    pd = {"u": (u, 3), "p": (p, 1)}
    cd = {"sigma": (sig, 9)}
    output.write_vtu(str(tmp_path / "a.vtu"), mesh.coords, mesh.tets, pd, cd)
    output.write_pvtu(str(tmp_path / "a.pvtu"), "a.vtu", pd, cd)
    root = ET.parse(tmp_path / "a.vtu").getroot()
    piece = root.find("UnstructuredGrid").find("Piece")
    assert int(piece.get("NumberOfPoints")) == mesh.num_nodes
    arrays = {a.get("Name"): a for a in piece.iter("DataArray")}
    assert np.array_equal(_decode(arrays["coordinates"].text, np.float64).reshape(-1, 3), mesh.coords)
    assert np.array_equal(_decode(arrays["connectivity"].text, np.int64).reshape(-1, 4), mesh.tets)
    assert np.array_equal(_decode(arrays["types"].text, np.uint8), np.full(mesh.num_elems, 10, np.uint8))
    assert np.array_equal(_decode(arrays["u"].text, np.float64).reshape(-1, 3), u)
    assert np.array_equal(_decode(arrays["sigma"].text, np.float64).reshape(-1, 9), sig)
    proot = ET.parse(tmp_path / "a.pvtu").getroot()
    assert proot.find("PUnstructuredGrid").find("Piece").get("Source") == "a.vtu"


def test_restart_round_trip(tmp_path):
    mesh = kuhn_cube(2)
    rng = np.random.default_rng(1)
    U = rng.standard_normal((mesh.num_nodes, 4))
    states = {"Fp": (rng.standard_normal((mesh.num_elems, 9)), 9), "eqps": (rng.random(mesh.num_elems), 1)}
    folder = tmp_path / "out_1"
    folder.mkdir()
    output.save_restart(str(folder / "restart.npz"), mesh, U, states)
    assert output.is_restart(str(folder))
    m2, U2, st2 = output.load_restart(str(folder))
    assert np.array_equal(m2.coords, mesh.coords) and np.array_equal(m2.tets, mesh.tets)
    assert m2.elem_set_names == mesh.elem_set_names
    for k in mesh.node_sets:
        assert np.array_equal(m2.node_sets[k], mesh.node_sets[k])
    for k in mesh.side_sets:
        assert np.array_equal(m2.side_sets[k], mesh.side_sets[k])
    assert np.array_equal(U2, U)
    assert np.array_equal(st2["Fp"], states["Fp"][0]) and np.array_equal(st2["eqps"], states["eqps"][0])
