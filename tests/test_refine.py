"""Conforming refinement to a target size (the refinement half of goal's
adaptation step) and the transfer onto the refined mesh. Host code, run on
the CPU: conformity (every interior face shared by exactly two tets, no
hanging node), volume and boundary area preserved, positive orientation,
midpoint coordinates, the size criterion met, node/side sets carried, and
determinism."""
import numpy as np

from goal_gb300 import adapt
from goal_gb300.mesh import kuhn_cube, graded_block


def _faces(tets):
    f = np.concatenate([tets[:, [1, 2, 3]], tets[:, [0, 3, 2]], tets[:, [0, 1, 3]], tets[:, [0, 2, 1]]])
    return np.sort(f, axis=1)


def _check_conforming(mesh):
    f = _faces(mesh.tets)
    _, counts = np.unique(f, axis=0, return_counts=True)
    assert counts.max() <= 2
    # boundary faces lie on the unit box's planes (no hanging faces inside)
    uniq, counts = np.unique(f, axis=0, return_counts=True)
    bnd = uniq[counts == 1]
    X = mesh.coords[bnd]
    lo, hi = mesh.coords.min(axis=0), mesh.coords.max(axis=0)
    on_plane = np.zeros(len(bnd), bool)
    for d in range(3):
        on_plane |= np.all(np.abs(X[:, :, d] - lo[d]) < 1e-12, axis=1)
        on_plane |= np.all(np.abs(X[:, :, d] - hi[d]) < 1e-12, axis=1)
    assert on_plane.all()
    return bnd


def _volumes(mesh):
    X = mesh.coords[mesh.tets]
    return np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0])) / 6.0


def _area(coords, tris):
    X = coords[tris]
    return 0.5 * np.linalg.norm(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), axis=1).sum()


def test_local_refinement_is_conforming():
    mesh = kuhn_cube(4)
    # fine near the corner (0, 0, 0), coarse elsewhere
    r = np.linalg.norm(mesh.coords, axis=1)
    size = 0.05 + 0.5 * r
    out, parents, origin = adapt.refine_to_size(mesh, size)
    assert out.num_elems > mesh.num_elems
    _check_conforming(out)
    v = _volumes(out)
    assert v.min() > 0
    assert abs(v.sum() - 1.0) < 1e-12
    # children tile their parents
    vp = np.bincount(origin, weights=v, minlength=mesh.num_elems)
    assert np.allclose(vp, _volumes(mesh), rtol=1e-12, atol=0)
    # new nodes at edge midpoints
    N = mesh.num_nodes
    assert np.allclose(out.coords[N:], 0.5 * (out.coords[parents[:, 0]] + out.coords[parents[:, 1]]), atol=0)
    # the size criterion holds everywhere
    s = adapt.transfer_nodal(size, parents)[:, 0]
    X = out.coords
    for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)):
        ea, eb = out.tets[:, a], out.tets[:, b]
        le = np.linalg.norm(X[ea] - X[eb], axis=1)
        assert np.all(le <= 1.5 * 0.5 * (s[ea] + s[eb]) * (1 + 1e-12))


def test_sets_and_boundary_area_are_carried():
    mesh = kuhn_cube(3)
    size = np.full(mesh.num_nodes, 0.12)
    out, parents, origin = adapt.refine_to_size(mesh, size)
    for name, tris in mesh.side_sets.items():
        assert abs(_area(out.coords, out.side_sets[name]) - _area(mesh.coords, tris)) < 1e-12
        # every side triangle is a boundary face of the refined mesh
        bnd = {tuple(f) for f in _check_conforming(out)}
        assert all(tuple(sorted(t)) in bnd for t in out.side_sets[name])
    for name, nodes in out.node_sets.items():
        d, v = {"xmin": (0, 0.0), "xmax": (0, 1.0), "ymin": (1, 0.0), "ymax": (1, 1.0), "zmin": (2, 0.0),
                "zmax": (2, 1.0)}[name]
        on = np.flatnonzero(np.abs(out.coords[:, d] - v) < 1e-12)
        assert np.array_equal(np.sort(nodes), on)


def test_deterministic_and_states_follow_parents():
    mesh = graded_block(1500, seed=4, regions=3)
    rng = np.random.default_rng(0)
    size = rng.uniform(0.05, 0.3, mesh.num_nodes)
    a = adapt.refine_to_size(mesh, size)
    b = adapt.refine_to_size(mesh, size)
    assert np.array_equal(a[0].tets, b[0].tets) and np.array_equal(a[0].coords, b[0].coords)
    out, parents, origin = a
    assert np.array_equal(out.elem_set, mesh.elem_set[origin])
    st = adapt.transfer_states({"eqps": np.arange(mesh.num_elems, dtype=float)}, origin)
    assert np.array_equal(st["eqps"], origin.astype(float))
    U = rng.standard_normal((mesh.num_nodes, 4))
    # a linear field is reproduced exactly at the new nodes
    lin = mesh.coords @ np.array([1.0, -2.0, 0.5]) + 3.0
    t = adapt.transfer_nodal(lin, parents)[:, 0]
    assert np.allclose(t, out.coords @ np.array([1.0, -2.0, 0.5]) + 3.0, atol=1e-12)
    assert adapt.transfer_nodal(U, parents).shape == (out.num_nodes, 4)


def test_cpp_mirror_refines(tmp_path):
    """goal::refine_to_size in the C++ mirror, compiled with g++ against the C
    ABI (the refiner is host code: no GPU needed)."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    from goal_gb300 import lib
    lib()  # built in-tree
    exe = tmp_path / "refine_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(root, "tests", "cpp", "refine_check.cpp"),
                           "-I", os.path.join(root, "include"), "-L", os.path.join(root, "goal_gb300"),
                           "-lgoal_gb300", f"-Wl,-rpath,{os.path.join(root, 'goal_gb300')}", "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
