"""Mesh adaptation to a target size field and the transfer of the solution
and states onto the adapted mesh: the adaptation step of goal's nested loop
(src/main_nested.cpp:106-126). goal remeshes with SCOREC ma::adapt (not part
of the reference); here the mesh is coarsened by edge collapse
(``goal_coarsener_*`` in the C ABI) and refined by conforming longest-edge
bisection (``goal_refiner_*``), driven by the isotropic target size field of
the DWR indicators (``api.size_field``, src/goal_size_field.cpp).

Transfer rules (the same as goal's nested-mesh rules, src/goal_nested.cpp:347-393):
a new node, at the midpoint of an edge, takes the mean of the edge's end
point values (exact for the linear fields); a child element takes its parent
element's integration-point states. A new node belongs to a node set when
both end points of its edge do; side triangles are split with their edges.
Coarsening keeps a subset of the nodes, which keep their values, and a subset
of the elements (with one node moved), which keep their states.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Tuple

import numpy as np

from . import lib
from .api import check, _f64, _i32, _ptr
from .mesh import Mesh


def refine_to_size(mesh: Mesh, vtx_size: np.ndarray, ratio: float = 1.5, max_elems: int = 50_000_000,
                   max_passes: int = 64) -> Tuple[Mesh, np.ndarray, np.ndarray]:
    """Refines until no edge is longer than ``ratio`` times the mean target
    size of its end points. Returns the refined mesh, the node parents
    (new nodes x 2, edge end points; new nodes follow the old ones) and the
    original element of every refined element."""
    L = lib()
    N, E = mesh.num_nodes, mesh.num_elems
    size = _f64(vtx_size)
    if size.shape != (N,):
        raise ValueError("one target size per node")
    names = sorted(mesh.side_sets)
    tris = [np.asarray(mesh.side_sets[k], np.int32).reshape(-1, 3) for k in names]
    tri = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 3), np.int32), dtype=np.int32)
    tri_set = np.ascontiguousarray(np.concatenate([np.full(len(t), i, np.int32) for i, t in enumerate(tris)])
                                   if tris else np.zeros(0, np.int32))
    h = ctypes.c_void_p()
    coords = _f64(mesh.coords)
    tets = _i32(mesh.tets)
    check(L.goal_refiner_create(N, _ptr(coords), E, _ptr(tets), len(tri), _ptr(tri), _ptr(tri_set), ctypes.byref(h)))
    try:
        sizes = (ctypes.c_longlong * 3)()
        check(L.goal_refiner_refine(h, _ptr(size), float(ratio), int(max_elems), int(max_passes), sizes))
        n2, e2, s2 = int(sizes[0]), int(sizes[1]), int(sizes[2])
        X = np.zeros((n2, 3))
        par = np.zeros((n2, 2), np.int32)
        T = np.zeros((e2, 4), np.int32)
        org = np.zeros(e2, np.int32)
        tri2 = np.zeros((s2, 3), np.int32)
        tset2 = np.zeros(s2, np.int32)
        check(L.goal_refiner_get(h, _ptr(X), _ptr(par), _ptr(T), _ptr(org), _ptr(tri2), _ptr(tset2)))
    finally:
        L.goal_refiner_destroy(h)
    new_parents = par[N:]
    node_sets = {}
    for name, nodes in mesh.node_sets.items():
        member = np.zeros(n2, bool)
        member[np.asarray(nodes, np.int64)] = True
        node_sets[name] = np.flatnonzero(_propagate(member, N, new_parents, np.logical_and)).astype(np.int32)
    side_sets = {name: tri2[tset2 == i] for i, name in enumerate(names)}
    out = Mesh(coords=X, tets=T, elem_set=np.asarray(mesh.elem_set)[org].astype(np.int32),
               elem_set_names=list(mesh.elem_set_names), node_sets=node_sets, side_sets=side_sets)
    return out, new_parents, org


def _node_class(mesh: Mesh) -> np.ndarray:
    """Per-node bit mask of node-set (bit k, k < 30) and side-set (bit 30 + k)
    memberships, for the coarsening rule that a collapsed node's sets are a
    subset of its target's."""
    cls = np.zeros(mesh.num_nodes, np.int64)
    for k, name in enumerate(sorted(mesh.node_sets)[:30]):
        cls[np.asarray(mesh.node_sets[name], np.int64)] |= np.int64(1) << k
    for k, name in enumerate(sorted(mesh.side_sets)[:30]):
        tri = np.asarray(mesh.side_sets[name], np.int64).reshape(-1)
        cls[np.unique(tri)] |= np.int64(1) << (30 + k)
    return cls


def coarsen_to_size(mesh: Mesh, vtx_size: np.ndarray, ratio: float = 0.5, refine_ratio: float = 1.5,
                    min_quality: float = 0.2, max_passes: int = 8) -> Tuple[Mesh, np.ndarray, np.ndarray]:
    """Collapses edges shorter than ``ratio`` times the mean target size of
    their end points (``goal_coarsener_*``: model and validity checks there).
    Returns the coarsened mesh, the original node of each kept node and the
    original element of each kept element."""
    L = lib()
    N, E = mesh.num_nodes, mesh.num_elems
    size = _f64(vtx_size)
    if size.shape != (N,):
        raise ValueError("one target size per node")
    names = sorted(mesh.side_sets)
    tris = [np.asarray(mesh.side_sets[k], np.int32).reshape(-1, 3) for k in names]
    tri = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 3), np.int32), dtype=np.int32)
    tri_set = np.ascontiguousarray(np.concatenate([np.full(len(t), i, np.int32) for i, t in enumerate(tris)])
                                   if tris else np.zeros(0, np.int32))
    coords = _f64(mesh.coords)
    tets = _i32(mesh.tets)
    eset = _i32(mesh.elem_set)
    cls = np.ascontiguousarray(_node_class(mesh))
    h = ctypes.c_void_p()
    check(L.goal_coarsener_create(N, _ptr(coords), E, _ptr(tets), _ptr(eset), _ptr(cls), len(tri), _ptr(tri),
                                  _ptr(tri_set), ctypes.byref(h)))
    try:
        sizes = (ctypes.c_longlong * 3)()
        check(L.goal_coarsener_coarsen(h, _ptr(size), float(ratio), float(refine_ratio), float(min_quality),
                                       int(max_passes), sizes))
        n2, e2, s2 = int(sizes[0]), int(sizes[1]), int(sizes[2])
        X = np.zeros((n2, 3))
        org_n = np.zeros(n2, np.int32)
        T = np.zeros((e2, 4), np.int32)
        org_e = np.zeros(e2, np.int32)
        tri2 = np.zeros((s2, 3), np.int32)
        tset2 = np.zeros(s2, np.int32)
        check(L.goal_coarsener_get(h, _ptr(X), _ptr(org_n), _ptr(T), _ptr(org_e), _ptr(tri2), _ptr(tset2)))
    finally:
        L.goal_coarsener_destroy(h)
    renum = np.full(N, -1, np.int64)
    renum[org_n] = np.arange(n2)
    node_sets = {}
    for name, nodes in mesh.node_sets.items():
        kept = renum[np.asarray(nodes, np.int64)]
        node_sets[name] = np.sort(kept[kept >= 0]).astype(np.int32)
    side_sets = {name: tri2[tset2 == i] for i, name in enumerate(names)}
    out = Mesh(coords=X, tets=T, elem_set=np.asarray(mesh.elem_set)[org_e].astype(np.int32),
               elem_set_names=list(mesh.elem_set_names), node_sets=node_sets, side_sets=side_sets)
    return out, org_n, org_e


def improve_shape(mesh: Mesh, target_quality: float = 0.3, max_passes: int = 4) -> Tuple[Mesh, np.ndarray]:
    """Flips (3-2 and 2-3, nodes fixed) around tets of mean-ratio quality
    below ``target_quality`` (``goal_coarsener_swap``). Returns the improved
    mesh and the original element of each element (the old tet that holds the
    new tet's centroid)."""
    L = lib()
    N, E = mesh.num_nodes, mesh.num_elems
    names = sorted(mesh.side_sets)
    tris = [np.asarray(mesh.side_sets[k], np.int32).reshape(-1, 3) for k in names]
    tri = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 3), np.int32), dtype=np.int32)
    tri_set = np.ascontiguousarray(np.concatenate([np.full(len(t), i, np.int32) for i, t in enumerate(tris)])
                                   if tris else np.zeros(0, np.int32))
    coords = _f64(mesh.coords)
    tets = _i32(mesh.tets)
    eset = _i32(mesh.elem_set)
    cls = np.ascontiguousarray(_node_class(mesh))
    h = ctypes.c_void_p()
    check(L.goal_coarsener_create(N, _ptr(coords), E, _ptr(tets), _ptr(eset), _ptr(cls), len(tri), _ptr(tri),
                                  _ptr(tri_set), ctypes.byref(h)))
    try:
        sizes = (ctypes.c_longlong * 3)()
        check(L.goal_coarsener_swap(h, float(target_quality), int(max_passes), sizes))
        n2, e2, s2 = int(sizes[0]), int(sizes[1]), int(sizes[2])
        X = np.zeros((n2, 3))
        org_n = np.zeros(n2, np.int32)
        T = np.zeros((e2, 4), np.int32)
        org_e = np.zeros(e2, np.int32)
        tri2 = np.zeros((s2, 3), np.int32)
        tset2 = np.zeros(s2, np.int32)
        check(L.goal_coarsener_get(h, _ptr(X), _ptr(org_n), _ptr(T), _ptr(org_e), _ptr(tri2), _ptr(tset2)))
    finally:
        L.goal_coarsener_destroy(h)
    side_sets = {name: tri2[tset2 == i] for i, name in enumerate(names)}
    out = Mesh(coords=X, tets=T, elem_set=np.asarray(mesh.elem_set)[org_e].astype(np.int32),
               elem_set_names=list(mesh.elem_set_names), node_sets=dict(mesh.node_sets), side_sets=side_sets)
    return out, org_e


def smooth(mesh: Mesh, target_quality: float = 0.3, max_passes: int = 4) -> Tuple[Mesh, Tuple[np.ndarray, ...]]:
    """Moves interior nodes (in no node or side set, inside one element set)
    of low-quality stars towards the mean of their neighbours
    (``goal_coarsener_smooth``). Returns the smoothed mesh and the nodal
    transfer as CSR rows (ptr, ids, weights) over the input mesh's nodes: a
    moved node takes the old field's value at its new position."""
    L = lib()
    N, E = mesh.num_nodes, mesh.num_elems
    names = sorted(mesh.side_sets)
    tris = [np.asarray(mesh.side_sets[k], np.int32).reshape(-1, 3) for k in names]
    tri = np.ascontiguousarray(np.concatenate(tris) if tris else np.zeros((0, 3), np.int32), dtype=np.int32)
    tri_set = np.ascontiguousarray(np.concatenate([np.full(len(t), i, np.int32) for i, t in enumerate(tris)])
                                   if tris else np.zeros(0, np.int32))
    coords = _f64(mesh.coords)
    tets = _i32(mesh.tets)
    eset = _i32(mesh.elem_set)
    cls = np.ascontiguousarray(_node_class(mesh))
    h = ctypes.c_void_p()
    check(L.goal_coarsener_create(N, _ptr(coords), E, _ptr(tets), _ptr(eset), _ptr(cls), len(tri), _ptr(tri),
                                  _ptr(tri_set), ctypes.byref(h)))
    try:
        nnz = ctypes.c_longlong()
        check(L.goal_coarsener_smooth(h, float(target_quality), int(max_passes), ctypes.byref(nnz)))
        X = np.zeros((N, 3))
        org_n = np.zeros(N, np.int32)
        T = np.zeros((E, 4), np.int32)
        org_e = np.zeros(E, np.int32)
        tri2 = np.zeros((len(tri), 3), np.int32)
        tset2 = np.zeros(len(tri), np.int32)
        check(L.goal_coarsener_get(h, _ptr(X), _ptr(org_n), _ptr(T), _ptr(org_e), _ptr(tri2), _ptr(tset2)))
        ptr = np.zeros(N + 1, np.int32)
        ids = np.zeros(nnz.value, np.int32)
        w = np.zeros(nnz.value)
        check(L.goal_coarsener_transfer(h, _ptr(ptr), _ptr(ids), _ptr(w)))
    finally:
        L.goal_coarsener_destroy(h)
    out = Mesh(coords=X, tets=T, elem_set=np.asarray(mesh.elem_set).astype(np.int32),
               elem_set_names=list(mesh.elem_set_names), node_sets=dict(mesh.node_sets),
               side_sets={name: tri2[tset2 == i] for i, name in enumerate(names)})
    return out, (ptr, ids, w)


def apply_rows(values: np.ndarray, rows: Tuple[np.ndarray, ...]) -> np.ndarray:
    """Nodal values through CSR transfer rows (ptr, ids, weights)."""
    ptr, ids, w = rows
    v = np.asarray(values, np.float64)
    v = v.reshape(len(v), -1)
    contrib = v[ids] * w[:, None]
    out = np.add.reduceat(contrib, ptr[:-1], axis=0) if len(ids) else np.zeros((len(ptr) - 1, v.shape[1]))
    return out


class Transfer:
    """Moves nodal fields and element states from the mesh before an
    adaptation to the mesh after it: through the coarsening (kept nodes keep
    their values, kept elements their states), then the refinement (midpoint
    means, children inherit)."""

    def __init__(self, node_origin: np.ndarray, elem_origin_c: np.ndarray, new_parents: np.ndarray,
                 elem_origin_r: np.ndarray, smooth_rows=None):
        self.node_origin = node_origin
        self.elem_origin_c = elem_origin_c
        self.new_parents = new_parents
        self.elem_origin_r = elem_origin_r
        self.smooth_rows = smooth_rows

    def nodal(self, values: np.ndarray) -> np.ndarray:
        v = np.asarray(values, np.float64)
        v = v.reshape(len(v), -1)[self.node_origin]
        if self.smooth_rows is not None:
            v = apply_rows(v, self.smooth_rows)
        return transfer_nodal(v, self.new_parents)

    def states(self, states: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
        return transfer_states(transfer_states(states, self.elem_origin_c), self.elem_origin_r)

    @property
    def elem_origin(self) -> np.ndarray:
        """The original element of every element of the adapted mesh."""
        return np.asarray(self.elem_origin_c)[self.elem_origin_r]


def adapt_to_size(mesh: Mesh, vtx_size: np.ndarray, coarsen_ratio: float = 0.5, refine_ratio: float = 1.5,
                  min_quality: float = 0.2, max_elems: int = 50_000_000,
                  improve_quality: float = 0.0) -> Tuple[Mesh, Transfer]:
    """One adaptation to a size field: coarsen (edges shorter than
    coarsen_ratio x size), optionally improve the tets of quality below
    improve_quality by flips and vertex smoothing (0: neither), then refine
    (edges longer than refine_ratio x size). Returns the adapted mesh and the
    transfer of fields onto it."""
    size = _f64(vtx_size)
    mc, org_n, org_ec = coarsen_to_size(mesh, size, ratio=coarsen_ratio, refine_ratio=refine_ratio,
                                        min_quality=min_quality)
    rows = None
    if improve_quality > 0.0:
        mc, org_f = improve_shape(mc, target_quality=improve_quality)
        org_ec = np.asarray(org_ec)[org_f]
        mc, rows = smooth(mc, target_quality=improve_quality)
    mr, parents, org_er = refine_to_size(mc, size[org_n], ratio=refine_ratio, max_elems=max_elems)
    return mr, Transfer(org_n, org_ec, parents, org_er, rows)


def _propagate(arr, base, new_parents, combine):
    """Fills arr[base:] from the parents (which precede their children) by
    sweeping all new nodes until nothing changes: one sweep per generation of
    bisection."""
    a, b = new_parents[:, 0], new_parents[:, 1]
    for _ in range(len(new_parents) + 1):
        nxt = combine(arr[a], arr[b])
        if np.array_equal(nxt, arr[base:]):
            break
        arr[base:] = nxt
    return arr


def transfer_nodal(values: np.ndarray, new_parents: np.ndarray) -> np.ndarray:
    """Nodal values (old nodes x c) on the refined mesh: a new node takes the
    mean of its edge's end points."""
    v = np.asarray(values, np.float64)
    v = v.reshape(len(v), -1)
    out = np.zeros((len(v) + len(new_parents), v.shape[1]))
    out[:len(v)] = v
    return _propagate(out, len(v), np.asarray(new_parents), lambda x, y: 0.5 * (x + y))


def transfer_states(states: Dict[str, np.ndarray], elem_origin: np.ndarray) -> Dict[str, np.ndarray]:
    """Element states on the refined mesh: every child takes its parent's."""
    return {k: np.asarray(v)[elem_origin] for k, v in states.items()}
