"""Coarsening by edge collapse (the coarsening half of goal's adaptation
step), shape improvement by 2-3 / 3-2 flips and vertex smoothing, and the coarsen-then-refine
adaptation with its field transfer. Host code, run on the CPU: conformity,
positive orientation, volume (per element set) and boundary area preserved,
boundary nodes and side sets kept on their planes, the length and quality
bounds, flips that pick the better of the two bipyramid configurations,
determinism, and exact transfer of a linear field."""
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


def _bipyramid(h, ring):
    """Triangle a b c on the unit circle (z = 0) and apexes d, e = (0, 0, -/+h):
    the two tets across face abc, or the three tets around edge de."""
    from goal_gb300.mesh import Mesh
    ang = np.array([0.0, 2.0, 4.0]) * np.pi / 3.0
    X = np.array([[np.cos(t), np.sin(t), 0.0] for t in ang] + [[0.0, 0.0, -h], [0.0, 0.0, h]])
    T = np.array([[0, 1, 3, 4], [1, 2, 3, 4], [2, 0, 3, 4]] if ring else [[0, 1, 2, 3], [0, 1, 2, 4]], np.int32)
    m = Mesh(coords=X, tets=T, elem_set=np.zeros(len(T), np.int32), elem_set_names=["b"], node_sets={},
             side_sets={})
    v = _volumes(m)
    m.tets[v < 0] = m.tets[v < 0][:, [0, 1, 3, 2]]
    return m


def test_flips_take_the_better_configuration():
    # flat bipyramid: three tets around the short axis beat two across the face
    m = _bipyramid(0.2, ring=False)
    out, origin = adapt.improve_shape(m, target_quality=0.6)
    assert out.num_elems == 3 and _volumes(out).min() > 0
    assert abs(_volumes(out).sum() - _volumes(m).sum()) < 1e-14
    assert _quality(out).min() > _quality(m).min() + 0.1
    assert set(origin) <= {0, 1}
    # tall bipyramid: two tets across the face beat the three around the axis
    m = _bipyramid(2.0, ring=True)
    out, origin = adapt.improve_shape(m, target_quality=0.6)
    assert out.num_elems == 2 and _volumes(out).min() > 0
    assert abs(_volumes(out).sum() - _volumes(m).sum()) < 1e-14
    assert _quality(out).min() > 0.9
    # good enough already: untouched
    m = _bipyramid(1.2, ring=False)
    out, origin = adapt.improve_shape(m, target_quality=0.6)
    assert np.array_equal(out.tets, m.tets) and np.array_equal(origin, [0, 1])


def test_flips_after_coarsening_keep_the_mesh_valid():
    mesh = kuhn_cube(10)
    mc, _, _ = adapt.coarsen_to_size(mesh, np.full(mesh.num_nodes, 0.35))
    out, origin = adapt.improve_shape(mc, target_quality=0.4)
    bnd = {tuple(f) for f in _check_conforming(out)}
    v = _volumes(out)
    assert v.min() > 0 and abs(v.sum() - 1.0) < 1e-12
    q0, q1 = _quality(mc), _quality(out)
    assert q1.min() >= q0.min() - 1e-12
    assert np.percentile(q1, 5) >= np.percentile(q0, 5) - 1e-12
    for name, (d, val) in PLANES.items():
        assert abs(_area(out.coords, out.side_sets[name]) - 1.0) < 1e-12
        assert all(tuple(sorted(t)) in bnd for t in out.side_sets[name])
    assert origin.min() >= 0 and origin.max() < mc.num_elems


def test_smoothing_raises_quality_and_moves_linear_fields_exactly():
    mesh = kuhn_cube(10, jitter=0.25, seed=3)
    out, rows = adapt.smooth(mesh, target_quality=0.35)
    assert np.array_equal(out.tets, mesh.tets)
    _check_conforming(out)
    v = _volumes(out)
    assert v.min() > 0 and abs(v.sum() - 1.0) < 1e-12
    q0, q1 = _quality(mesh), _quality(out)
    assert q1.min() > q0.min() + 0.05
    moved = np.any(out.coords != mesh.coords, axis=1)
    assert moved.sum() > 0
    # boundary and set nodes stay put
    for name, nodes in mesh.node_sets.items():
        assert not moved[nodes].any()
    # a linear field moves exactly; unmoved nodes keep their values
    g = np.array([1.0, -2.0, 0.5])
    lin = np.stack([mesh.coords @ g + 3.0, mesh.coords[:, 2]], axis=1)
    t = adapt.apply_rows(lin, rows)
    assert np.allclose(t[:, 0], out.coords @ g + 3.0, atol=1e-12)
    assert np.allclose(t[:, 1], out.coords[:, 2], atol=1e-12)
    assert np.array_equal(t[~moved], lin[~moved])


def test_adapt_with_shape_improvement():
    mesh = kuhn_cube(8, jitter=0.2, seed=1)
    r = np.linalg.norm(mesh.coords, axis=1)
    size = 0.05 + 0.4 * r
    out, tr = adapt.adapt_to_size(mesh, size, improve_quality=0.35)
    _check_conforming(out)
    v = _volumes(out)
    assert v.min() > 0 and abs(v.sum() - 1.0) < 1e-12
    g = np.array([0.3, 1.0, -0.7])
    t = tr.nodal(mesh.coords @ g)
    assert np.allclose(t[:, 0], out.coords @ g, atol=1e-12)
    st = tr.states({"eqps": np.arange(mesh.num_elems, dtype=float)})
    assert st["eqps"].shape == (out.num_elems,)


def test_bad_arguments_are_errors():
    import ctypes
    from goal_gb300 import lib
    from goal_gb300.api import GoalError, check
    L = lib()
    h = ctypes.c_void_p()
    X = np.zeros(12)
    T = np.array([0, 1, 2, 4], np.int32)  # node 4 of 4
    cls = np.zeros(4, np.int64)
    rc = L.goal_coarsener_create(4, X.ctypes.data, 1, T.ctypes.data, None, cls.ctypes.data, 0, None, None,
                                 ctypes.byref(h))
    assert rc != 0
    try:
        check(rc)
        raise AssertionError("expected an error")
    except GoalError as e:
        assert "out of range" in str(e)
    mesh = kuhn_cube(2)
    with np.testing.assert_raises(Exception):
        adapt.coarsen_to_size(mesh, np.zeros(mesh.num_nodes))  # sizes must be positive
    with np.testing.assert_raises(ValueError):
        adapt.coarsen_to_size(mesh, np.ones(3))
