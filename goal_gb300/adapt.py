"""Mesh refinement to a target size field and the transfer of the solution
and states onto the refined mesh: the adaptation step of goal's nested loop
(src/main_nested.cpp:106-126). goal remeshes with SCOREC ma::adapt (not part
of the reference); here the mesh is refined by conforming longest-edge
bisection (``goal_refiner_*`` in the C ABI), driven by the isotropic target
size field of the DWR indicators (``api.size_field``, src/goal_size_field.cpp).

Transfer rules (the same as goal's nested-mesh rules, src/goal_nested.cpp:347-393):
a new node, at the midpoint of an edge, takes the mean of the edge's end
point values (exact for the linear fields); a child element takes its parent
element's integration-point states. A new node belongs to a node set when
both end points of its edge do; side triangles are split with their edges.
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
