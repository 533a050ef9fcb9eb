"""Reader for the discretization inputs goal loads: a SCOREC SMB v5 mesh (one
part file, or the part files of a partitioned mesh), its ``.dmg`` model and
the association file (src/goal_disc.cpp:28-120).

File names follow SCOREC's convention: a mesh file ``name.smb`` is stored as
part files ``name0.smb``, ``name1.smb``, ... (one per MPI rank of the run that
wrote it; ``cube.smb`` of the reference's 3D test is ``cube0.smb`` to
``cube3.smb``, and ``cube-serial.smb`` is ``cube-serial0.smb``). Every part
is read and the parts are joined into one mesh: part-boundary vertices appear
in every part that holds them, with the same coordinates, and are merged.

Only what the element path needs is decoded: vertex coordinates, tets (from
the tet->triangle->edge->vertex downward chain) and the (model tag, model dim)
classification of every entity. Sets follow goal's rules:

* elem set  -> tets classified on the listed model regions;
* side set  -> triangles classified on the listed model faces
  (``Disc::compute_side_sets``, src/goal_disc.cpp:362-377);
* node set  -> vertices whose classification, or any model entity above it in
  the model's upward adjacency, is a listed model entity
  (``apf::collectEntityModels`` as used by ``Disc::compute_node_sets``,
  src/goal_disc.cpp:379-396).

Tets are returned positively oriented. Node numbering is the file's vertex
order (goal renumbers with ``apf::reorderMdsMesh``; assembled quantities do not
depend on the numbering).
"""
from __future__ import annotations

import os
import struct
from typing import Dict, List, Tuple

import numpy as np

from .mesh import Mesh, orient_positive

# SMB entity type order in the file header: vertex, edge, triangle, quad,
# hex, prism, pyramid, tet.
_SMB_VERT, _SMB_EDGE, _SMB_TRI, _SMB_QUAD, _SMB_HEX, _SMB_PRISM, _SMB_PYR, _SMB_TET = range(8)


def read_smb(path: str):
    """Returns (coords (N,3), edges (NE,2), tris (NT,3 edge ids), tets (NTet,4 tri ids),
    classification dict type -> (n,2) [tag, dim])."""
    with open(path, "rb") as f:
        data = f.read()
    off = 0

    def ints(n):
        nonlocal off
        v = np.frombuffer(data, dtype=">u4", count=n, offset=off).astype(np.int64)
        off += 4 * n
        return v

    magic, version, dim, nparts = ints(4)
    if magic != 0 or version != 5:
        raise ValueError(f"{path}: not an SMB v5 file (magic {magic}, version {version})")
    if dim != 3:
        raise ValueError(f"{path}: only 3D meshes are supported (dim {dim})")
    counts = ints(8)
    if counts[_SMB_QUAD] or counts[_SMB_HEX] or counts[_SMB_PRISM] or counts[_SMB_PYR]:
        raise ValueError(f"{path}: only simplex meshes are supported")
    nv, ne, nt, ntet = (int(counts[_SMB_VERT]), int(counts[_SMB_EDGE]),
                        int(counts[_SMB_TRI]), int(counts[_SMB_TET]))
    edges = ints(2 * ne).reshape(ne, 2)
    tris = ints(3 * nt).reshape(nt, 3)
    tets = ints(4 * ntet).reshape(ntet, 4)
    coords = np.frombuffer(data, dtype=">f8", count=3 * nv, offset=off).astype(np.float64).reshape(nv, 3)
    off += 8 * 3 * nv
    off += 8 * 2 * nv  # parametric coordinates of vertices (unused)
    # remote copies: the number of peer parts, their ids, the number of
    # vertices shared with each, then those vertices' local ids (zero peers
    # in a one-part mesh); the join matches shared vertices by coordinates
    npeers = int(ints(1)[0])
    if npeers:
        ints(npeers)
        shared = ints(npeers)
        ints(int(shared.sum()))
    cls = {}
    for t, n in ((_SMB_VERT, nv), (_SMB_EDGE, ne), (_SMB_TRI, nt), (_SMB_TET, ntet)):
        cls[t] = ints(2 * n).reshape(n, 2)
    return coords, edges, tris, tets, cls


def read_dmg(path: str):
    """Model topology: dict dim -> {tag: [adjacent tags of dim-1]} plus the
    upward adjacency dict dim -> {tag: [tags of dim+1]}."""
    with open(path) as f:
        tok = f.read().split()
    it = iter(tok)
    nr, nf, ne, nv = (int(next(it)) for _ in range(4))
    for _ in range(6):
        next(it)
    down: Dict[int, Dict[int, List[int]]] = {0: {}, 1: {}, 2: {}, 3: {}}
    for _ in range(nv):
        tag = int(next(it)); next(it); next(it); next(it)
        down[0][tag] = []
    for _ in range(ne):
        tag = int(next(it)); a = int(next(it)); b = int(next(it))
        down[1][tag] = [a, b]
    for dim, count in ((2, nf), (3, nr)):
        for _ in range(count):
            tag = int(next(it)); nloops = int(next(it))
            ents = []
            for _ in range(nloops):
                n = int(next(it))
                for _ in range(n):
                    ents.append(int(next(it))); next(it)
            down[dim][tag] = ents
    up: Dict[int, Dict[int, List[int]]] = {0: {}, 1: {}, 2: {}, 3: {}}
    for dim in (1, 2, 3):
        for tag, below in down[dim].items():
            for b in below:
                up[dim - 1].setdefault(b, []).append(tag)
    return down, up


def read_assoc(path: str) -> List[Tuple[str, str, List[Tuple[int, int]]]]:
    """[(kind, name, [(model dim, model tag), ...])] with kind in
    {'node set', 'side set', 'elem set'} (src/goal_disc.cpp:28-73)."""
    out = []
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    i = 0
    while i < len(lines) and lines[i]:
        ln = lines[i]
        kind = None
        for k in ("node set", "side set", "elem set"):
            if ln.startswith(k):
                kind = k
        if kind is None:
            raise ValueError(f"invalid association line {i + 1}: {ln}")
        name, n = ln[len(kind):].split()
        ents = []
        for j in range(int(n)):
            d, t = lines[i + 1 + j].split()
            ents.append((int(d), int(t)))
        out.append((kind, name, ents))
        i += 1 + int(n)
    return out


def part_files(mesh_file: str) -> List[str]:
    """The part files of a mesh file name: ``name.smb`` itself if it exists,
    else ``name0.smb``, ``name1.smb``, ... as far as they exist."""
    if os.path.exists(mesh_file):
        return [mesh_file]
    stem = mesh_file[:-4] if mesh_file.endswith(".smb") else mesh_file
    out = []
    while os.path.exists(f"{stem}{len(out)}.smb"):
        out.append(f"{stem}{len(out)}.smb")
    if not out:
        raise FileNotFoundError(f"no SMB part files for {mesh_file} ({stem}0.smb, ...)")
    return out


def _vertices(coords, edges, tris, tets):
    """Vertices of every triangle (from its edges) and tet (from its triangles)."""
    tri_verts = np.empty((tris.shape[0], 3), np.int64)
    for t in range(tris.shape[0]):
        vs = []
        for e in tris[t]:
            for v in edges[e]:
                if v not in vs:
                    vs.append(v)
        tri_verts[t] = vs
    tet_verts = np.empty((tets.shape[0], 4), np.int64)
    for t in range(tets.shape[0]):
        vs = list(tri_verts[tets[t, 0]])
        for f in tets[t, 1:]:
            for v in tri_verts[f]:
                if v not in vs:
                    vs.append(v)
        if len(vs) != 4:
            raise ValueError("degenerate tet in SMB file")
        tet_verts[t] = vs
    return tri_verts, tet_verts


def read_parts(mesh_file: str):
    """Reads every part of a mesh and joins them: (coords, tri_verts,
    tet_verts, vertex / triangle / tet classification). Vertices shared by
    parts are merged by coordinates; triangles on part boundaries are kept once."""
    coords_all, vcls_all, tri_all, tcls_all, tet_all, ecls_all = [], [], [], [], [], []
    key_to_id: Dict[Tuple[float, float, float], int] = {}
    seen_tris = set()
    for path in part_files(mesh_file):
        coords, edges, tris, tets, cls = read_smb(path)
        tri_verts, tet_verts = _vertices(coords, edges, tris, tets)
        gid = np.empty(coords.shape[0], np.int64)
        for v in range(coords.shape[0]):
            key = tuple(coords[v])
            g = key_to_id.get(key)
            if g is None:
                g = len(coords_all)
                key_to_id[key] = g
                coords_all.append(coords[v])
                vcls_all.append(cls[_SMB_VERT][v])
            gid[v] = g
        for t in range(tri_verts.shape[0]):
            g = gid[tri_verts[t]]
            k = tuple(sorted(g))
            if k in seen_tris:
                continue
            seen_tris.add(k)
            tri_all.append(g)
            tcls_all.append(cls[_SMB_TRI][t])
        tet_all.append(gid[tet_verts])
        ecls_all.append(cls[_SMB_TET])
    coords = np.array(coords_all, dtype=np.float64).reshape(-1, 3)
    cls = {_SMB_VERT: np.array(vcls_all).reshape(-1, 2), _SMB_TRI: np.array(tcls_all).reshape(-1, 2),
           _SMB_TET: np.concatenate(ecls_all).reshape(-1, 2)}
    return coords, np.array(tri_all, np.int64).reshape(-1, 3), np.concatenate(tet_all).reshape(-1, 4), cls


def load(geom_file: str, mesh_file: str, assoc_file: str) -> Mesh:
    coords, tri_verts, tet_verts, cls = read_parts(mesh_file)
    _, up = read_dmg(geom_file)
    assoc = read_assoc(assoc_file)
    tet_verts = orient_positive(coords, tet_verts.astype(np.int32))

    def closure_up(dim, tag):
        seen = {(dim, tag)}
        stack = [(dim, tag)]
        while stack:
            d, t = stack.pop()
            for u in up.get(d, {}).get(t, []):
                if (d + 1, u) not in seen:
                    seen.add((d + 1, u))
                    stack.append((d + 1, u))
        return seen

    elem_set_names: List[str] = []
    elem_set = np.full(tet_verts.shape[0], -1, np.int32)
    node_sets: Dict[str, np.ndarray] = {}
    side_sets: Dict[str, np.ndarray] = {}
    vcls = cls[_SMB_VERT]
    vclosure = [closure_up(int(vcls[v, 1]), int(vcls[v, 0])) for v in range(coords.shape[0])]
    for kind, name, ents in assoc:
        ents_set = set(ents)
        if kind == "elem set":
            idx = len(elem_set_names)
            elem_set_names.append(name)
            c = cls[_SMB_TET]
            for t in range(tet_verts.shape[0]):
                if (int(c[t, 1]), int(c[t, 0])) in ents_set:
                    elem_set[t] = idx
        elif kind == "side set":
            c = cls[_SMB_TRI]
            sel = [t for t in range(tri_verts.shape[0]) if (int(c[t, 1]), int(c[t, 0])) in ents_set]
            side_sets[name] = np.ascontiguousarray(tri_verts[sel], dtype=np.int32).reshape(-1, 3)
        else:
            sel = [v for v in range(coords.shape[0]) if vclosure[v] & ents_set]
            node_sets[name] = np.array(sel, dtype=np.int32)
    if (elem_set < 0).any():
        raise ValueError("tets not covered by any element set")
    return Mesh(coords=np.ascontiguousarray(coords), tets=tet_verts, elem_set=elem_set,
                elem_set_names=elem_set_names, node_sets=node_sets, side_sets=side_sets)
