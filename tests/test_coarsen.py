"""Coarsening by edge collapse (the coarsening half of goal's adaptation
step) and the coarsen-then-refine adaptation with its field transfer. Host
code, run on the CPU: conformity, positive orientation, volume (per element
set) and boundary area preserved, boundary nodes and side sets kept on their
planes, the length and quality bounds, determinism, and exact transfer of a
linear field."""
import numpy as np

from goal_gb300 import adapt
from goal_gb300.mesh import kuhn_cube, graded_block

from test_refine import _area, _check_conforming, _volumes

EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))
PLANES = {"xmin": (0, 0.0), "xmax": (0, 1.0), "ymin": (1, 0.0), "ymax": (1, 1.0), "zmin": (2, 0.0), "zmax": (2, 1.0)}


def _quality(mesh):
    X = mesh.coords[mesh.tets]
    V = _volumes(mesh)
    l2 = sum(np.sum((X[:, a] - X[:, b]) ** 2, axis=1) for a, b in EDGES)
    return 12.0 * np.cbrt(9.0 * V * V) / l2


def _edge_ratio(mesh, size):
    X = mesh.coords
    r = []
    for a, b in EDGES:
        ea, eb = mesh.tets[:, a], mesh.tets[:, b]
        r.append(np.linalg.norm(X[ea] - X[eb], axis=1) / (0.5 * (size[ea] + size[eb])))
    return np.concatenate(r)


def test_uniform_coarsening_is_valid():
    mesh = kuhn_cube(8)
    size = np.full(mesh.num_nodes, 0.4)
    out, node_origin, elem_origin = adapt.coarsen_to_size(mesh, size)
    assert out.num_elems < 0.5 * mesh.num_elems
    bnd = _check_conforming(out)
    v = _volumes(out)
    assert v.min() > 0 and abs(v.sum() - 1.0) < 1e-12
    # the box's surface: six unit faces
    assert abs(_area(out.coords, bnd) - 6.0) < 1e-12
    # kept nodes keep their coordinates; kept elements stay in order
    assert np.array_equal(out.coords, mesh.coords[node_origin])
    assert np.all(np.diff(node_origin) > 0) and np.all(np.diff(elem_origin) > 0)
    # no edge longer than the refinement threshold, quality bound
    assert _edge_ratio(out, size[node_origin]).max() <= 1.5 * (1 + 1e-12)
    assert _quality(out).min() >= min(0.2, _quality(mesh).min()) - 1e-12


def test_sets_stay_on_their_planes():
    mesh = kuhn_cube(6)
    size = np.full(mesh.num_nodes, 0.35)
    out, node_origin, _ = adapt.coarsen_to_size(mesh, size)
    bnd = {tuple(f) for f in _check_conforming(out)}
    for name, (d, val) in PLANES.items():
        nodes = out.node_sets[name]
        on = np.flatnonzero(np.abs(out.coords[:, d] - val) < 1e-12)
        assert np.array_equal(np.sort(nodes), on)
        tris = out.side_sets[name]
        assert abs(_area(out.coords, tris) - 1.0) < 1e-12
        assert np.all(np.abs(out.coords[tris][:, :, d] - val) < 1e-12)
        assert all(tuple(sorted(t)) in bnd for t in tris)
    # the box's corners and edges survive
    for c in np.array(np.meshgrid([0, 1], [0, 1], [0, 1])).T.reshape(-1, 3):
        assert np.any(np.all(np.abs(out.coords - c) < 1e-12, axis=1))


def test_element_sets_keep_their_volume_and_deterministic():
    mesh = graded_block(3000, seed=2, regions=4)
    rng = np.random.default_rng(1)
    size = rng.uniform(0.3, 0.6, mesh.num_nodes)
    a = adapt.coarsen_to_size(mesh, size)
    b = adapt.coarsen_to_size(mesh, size)
    assert np.array_equal(a[0].tets, b[0].tets) and np.array_equal(a[0].coords, b[0].coords)
    out, node_origin, elem_origin = a
    assert out.num_elems < mesh.num_elems
    _check_conforming(out)
    v0, v1 = _volumes(mesh), _volumes(out)
    assert v1.min() > 0
    for k in range(len(mesh.elem_set_names)):
        assert abs(v1[out.elem_set == k].sum() - v0[mesh.elem_set == k].sum()) < 1e-12
    assert np.array_equal(out.elem_set, mesh.elem_set[elem_origin])


def test_adapt_coarsens_and_refines_with_exact_linear_transfer():
    mesh = kuhn_cube(8)
    # fine near the corner (0, 0, 0), coarser than the mesh elsewhere
    r = np.linalg.norm(mesh.coords, axis=1)
    size = 0.04 + 0.4 * r
    out, tr = adapt.adapt_to_size(mesh, size)
    _check_conforming(out)
    v = _volumes(out)
    assert v.min() > 0 and abs(v.sum() - 1.0) < 1e-12
    near = np.linalg.norm(out.coords[out.tets].mean(axis=1), axis=1)
    near0 = np.linalg.norm(mesh.coords[mesh.tets].mean(axis=1), axis=1)
    # more elements than before near the corner, fewer far from it
    assert np.sum(near < 0.25) > np.sum(near0 < 0.25)
    assert np.sum(near > 0.9) < np.sum(near0 > 0.9)
    # a linear field moves exactly; states follow the original elements
    g = np.array([1.0, -2.0, 0.5])
    lin = np.stack([mesh.coords @ g + 3.0, mesh.coords[:, 0]], axis=1)
    t = tr.nodal(lin)
    assert np.allclose(t[:, 0], out.coords @ g + 3.0, atol=1e-12)
    assert np.allclose(t[:, 1], out.coords[:, 0], atol=1e-12)
    st = tr.states({"eqps": np.arange(mesh.num_elems, dtype=float)})
    assert np.array_equal(st["eqps"], tr.elem_origin.astype(float))
    assert np.array_equal(out.elem_set, mesh.elem_set[tr.elem_origin])


def test_nothing_to_collapse_is_identity():
    mesh = kuhn_cube(4)
    size = np.full(mesh.num_nodes, 0.25)  # h / size = 1: no edge below half the size
    out, node_origin, elem_origin = adapt.coarsen_to_size(mesh, size)
    assert np.array_equal(out.tets, mesh.tets) and np.array_equal(out.coords, mesh.coords)
    assert np.array_equal(node_origin, np.arange(mesh.num_nodes))
    assert np.array_equal(elem_origin, np.arange(mesh.num_elems))
