"""Linear-tet meshes with named element, node and side sets.

The host-side description of a discretization that ``Disc`` (goal_disc.hpp)
reads from SCOREC files: coordinates, tet connectivity, element sets, node
sets (nodes on the closure of model entities, src/goal_disc.cpp:379-396) and
side sets (boundary triangles, src/goal_disc.cpp:362-377).

Also the synthetic generators used for the benchmark workloads:

* ``kuhn_cube(n)``: [0,1]^3 split into n^3 hexes, each cut into 6 tets sharing
  the hex's main diagonal (E = 6 n^3, N = (n+1)^3).
* ``graded_block(...)``: a 4x1x1 block with a seeded smooth size field
  (three Gaussian bumps), tet count set by a target.
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, List

import numpy as np


@dataclasses.dataclass
class Mesh:
    coords: np.ndarray                 # (N, 3) float64
    tets: np.ndarray                   # (E, 4) int32, positively oriented
    elem_set: np.ndarray               # (E,) int32 index into elem_set_names
    elem_set_names: List[str]
    node_sets: Dict[str, np.ndarray]   # name -> sorted int32 node ids
    side_sets: Dict[str, np.ndarray]   # name -> (S, 3) int32 triangles

    @property
    def num_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def num_elems(self) -> int:
        return int(self.tets.shape[0])

    def volumes(self) -> np.ndarray:
        x = self.coords
        t = self.tets
        a = x[t[:, 1]] - x[t[:, 0]]
        b = x[t[:, 2]] - x[t[:, 0]]
        c = x[t[:, 3]] - x[t[:, 0]]
        return np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0


def orient_positive(coords: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Swap the last two vertices of every negatively oriented tet."""
    tets = np.ascontiguousarray(tets, dtype=np.int32).copy()
    x = coords
    a = x[tets[:, 1]] - x[tets[:, 0]]
    b = x[tets[:, 2]] - x[tets[:, 0]]
    c = x[tets[:, 3]] - x[tets[:, 0]]
    vol = np.einsum("ij,ij->i", a, np.cross(b, c))
    neg = vol < 0
    tmp = tets[neg, 2].copy()
    tets[neg, 2] = tets[neg, 3]
    tets[neg, 3] = tmp
    return tets


def boundary_faces_on(coords: np.ndarray, tets: np.ndarray, mask_nodes: np.ndarray) -> np.ndarray:
    """Tet faces whose three nodes all satisfy ``mask_nodes`` (boundary planes)."""
    faces = []
    for omit in range(4):
        keep = [k for k in range(4) if k != omit]
        f = tets[:, keep]
        on = mask_nodes[f].all(axis=1)
        faces.append(f[on])
    if not faces:
        return np.zeros((0, 3), np.int32)
    return np.ascontiguousarray(np.concatenate(faces, axis=0), dtype=np.int32)


def _plane_sets(coords: np.ndarray, tets: np.ndarray, lo: np.ndarray, hi: np.ndarray, tol: float):
    names = ["x", "y", "z"]
    node_sets = {}
    side_sets = {}
    for d in range(3):
        for tag, val in (("min", lo[d]), ("max", hi[d])):
            on = np.abs(coords[:, d] - val) <= tol
            node_sets[names[d] + tag] = np.nonzero(on)[0].astype(np.int32)
            side_sets[names[d] + tag] = boundary_faces_on(coords, tets, on)
    return node_sets, side_sets


def kuhn_cube(n: int, length=(1.0, 1.0, 1.0), set_name: str = "cube", jitter: float = 0.0, seed: int = 0) -> Mesh:
    """Structured n x n x n hex grid of [0,Lx]x[0,Ly]x[0,Lz], 6 Kuhn tets per hex.

    jitter > 0 moves every interior node by a seeded uniform offset in
    [-jitter, jitter] x (grid spacing) per coordinate, which removes the
    translation symmetry of the grid (boundary nodes stay on their faces);
    jitter <= 0.25 keeps every tet positively oriented."""
    n1 = n + 1
    g = np.arange(n1, dtype=np.float64) / n
    X, Y, Z = np.meshgrid(g * length[0], g * length[1], g * length[2], indexing="ij")
    # node id = i + n1*(j + n1*k)
    coords = np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(), Z.transpose(2, 1, 0).ravel()], axis=1)
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    step = [1, n1, n1 * n1]
    base = i + n1 * (j + n1 * k)
    tets = []
    for perm in itertools.permutations(range(3)):
        v0 = base
        v1 = v0 + step[perm[0]]
        v2 = v1 + step[perm[1]]
        v3 = v2 + step[perm[2]]
        tets.append(np.stack([v0, v1, v2, v3], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    tets = orient_positive(coords, tets)
    node_sets, side_sets = _plane_sets(coords, tets, np.zeros(3), np.array(length, float), 1e-12)
    if jitter > 0.0:
        if jitter > 0.25:
            raise ValueError("jitter above 0.25 can invert tets")
        L = np.array(length, float)
        interior = np.all((coords > 1e-12 * L) & (coords < L - 1e-12 * L), axis=1)
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=coords.shape) * (L / n)
        coords = coords + d * interior[:, None]
    return Mesh(coords=np.ascontiguousarray(coords), tets=tets,
                elem_set=np.zeros(tets.shape[0], np.int32), elem_set_names=[set_name],
                node_sets=node_sets, side_sets=side_sets)


def graded_block(target_elems: int, seed: int = 0, h_ratio: float = 8.0, set_name: str = "block",
                 regions: int = 1) -> Mesh:
    """4x1x1 block meshed with Kuhn tets on a tensor grid graded by a smooth
    seeded size field made of three Gaussian bumps (h ratio up to ``h_ratio``).

    The grading is separable (one 1-D spacing per axis, each the marginal of
    the 3-D size field), so the mesh stays a conforming Kuhn triangulation.
    regions > 1 splits the block into that many element sets ("region<i>"),
    the Voronoi cells of seeded points, for piecewise-constant materials.
    """
    rng = np.random.default_rng(seed)
    centers = rng.uniform([0.0, 0.0, 0.0], [4.0, 1.0, 1.0], size=(3, 3))
    widths = rng.uniform(0.15, 0.4, size=3)

    def size(x, d):
        # relative element size along axis d at coordinate x (1 = coarsest)
        s = np.ones_like(x)
        for c, w in zip(centers, widths):
            s = s - (1.0 - 1.0 / h_ratio) * np.exp(-0.5 * ((x - c[d]) / w) ** 2)
        return np.clip(s, 1.0 / h_ratio, 1.0)

    lengths = np.array([4.0, 1.0, 1.0])
    # choose base counts so that 6 * nx * ny * nz ~ target
    fine = 2048
    dens = []
    for d in range(3):
        xs = np.linspace(0.0, lengths[d], fine)
        dens.append(1.0 / size(xs, d))
    ints = [np.trapezoid(dens[d], np.linspace(0.0, lengths[d], fine)) for d in range(3)]
    scale = (target_elems / 6.0 / (ints[0] * ints[1] * ints[2])) ** (1.0 / 3.0)
    axes = []
    for d in range(3):
        xs = np.linspace(0.0, lengths[d], fine)
        cdf = np.concatenate([[0.0], np.cumsum(0.5 * (dens[d][1:] + dens[d][:-1]) * np.diff(xs))])
        m = max(1, int(round(scale * cdf[-1])))
        targets = np.linspace(0.0, cdf[-1], m + 1)
        axes.append(np.interp(targets, cdf, xs))
    nx, ny, nz = (len(a) - 1 for a in axes)
    X, Y, Z = np.meshgrid(axes[0], axes[1], axes[2], indexing="ij")
    coords = np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(), Z.transpose(2, 1, 0).ravel()], axis=1)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    step = [1, nx + 1, (nx + 1) * (ny + 1)]
    base = i + (nx + 1) * (j + (ny + 1) * k)
    tets = []
    for perm in itertools.permutations(range(3)):
        v0 = base
        v1 = v0 + step[perm[0]]
        v2 = v1 + step[perm[1]]
        v3 = v2 + step[perm[2]]
        tets.append(np.stack([v0, v1, v2, v3], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    tets = orient_positive(coords, tets)
    node_sets, side_sets = _plane_sets(coords, tets, np.zeros(3), lengths, 1e-12)
    elem_set = np.zeros(tets.shape[0], np.int32)
    names = [set_name]
    if regions > 1:
        pts = rng.uniform([0.0, 0.0, 0.0], lengths, size=(regions, 3))
        cent = coords[tets].mean(axis=1)
        d2 = ((cent[:, None, :] - pts[None, :, :]) ** 2).sum(axis=2)
        elem_set = np.argmin(d2, axis=1).astype(np.int32)
        names = [f"region{i}" for i in range(regions)]
    return Mesh(coords=np.ascontiguousarray(coords), tets=tets, elem_set=elem_set, elem_set_names=names,
                node_sets=node_sets, side_sets=side_sets)


def save_npz(mesh: Mesh, path: str) -> None:
    arrays = dict(coords=mesh.coords, tets=mesh.tets, elem_set=mesh.elem_set)
    for k, v in mesh.node_sets.items():
        arrays["ns_" + k] = v
    for k, v in mesh.side_sets.items():
        arrays["ss_" + k] = v
    np.savez(path, **arrays)


def load_npz(path: str, elem_set_names=None) -> Mesh:
    z = np.load(path)
    node_sets = {k[3:]: np.ascontiguousarray(z[k], dtype=np.int32) for k in z.files if k.startswith("ns_")}
    side_sets = {k[3:]: np.ascontiguousarray(z[k], dtype=np.int32).reshape(-1, 3) for k in z.files if k.startswith("ss_")}
    es = np.ascontiguousarray(z["elem_set"], dtype=np.int32)
    names = elem_set_names or ["set%d" % i for i in range(int(es.max()) + 1)]
    return Mesh(coords=np.ascontiguousarray(z["coords"], dtype=np.float64),
                tets=np.ascontiguousarray(z["tets"], dtype=np.int32), elem_set=es,
                elem_set_names=names, node_sets=node_sets, side_sets=side_sets)
