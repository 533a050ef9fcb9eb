"""Python side of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_build/liboracle.so (built from oracle/oracle.cpp by ``build()``)
and drives it the way goal's host drivers drive assemble():

* ``Primal.solve``     -- Newton loop of src/goal_primal.cpp:111-137 with the
  jacobian chain (src/goal_primal.cpp:92-109) and residual chain
  (src/goal_primal.cpp:75-90); linear systems solved directly with SciPy
  (the reference's GMRES/AMG converges to the same Newton iterates within its
  1e-10 relative linear tolerance).
* ``functional``       -- Functional::compute (src/goal_functional.cpp:62-70).
* ``nested_adjoint``   -- NestedAdjoint::run (src/goal_nested_adjoint.cpp:163-257)
  on the uniformly refined mesh produced by ``refine_uniform`` (the declared
  refinement rule shared with the CUDA path).

Only tests/, the smoke check and bench.py's CPU-baseline leg import this.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

NONE, PRIMAL, ADJOINT = 0, 1, 2
NEOHOOKEAN, J2 = 0, 1
QOI_NONE, QOI_AVG_DISP, QOI_KS = 0, 1, 2


TUNED_LIB = os.path.join(BUILD, "libtuned.so")


def build(force: bool = False) -> str:
    """Compile the C++ restatement (plain g++, no FMA contraction, so x86 and
    Arm hosts give the same bits) and the tuned CPU baseline (tuned.cpp)."""
    os.makedirs(BUILD, exist_ok=True)
    for src, lib, flags in ((os.path.join(HERE, "oracle.cpp"), LIB, ["-O2", "-ffp-contract=off"]),
                            (os.path.join(HERE, "tuned.cpp"), TUNED_LIB, ["-O3"])):
        if force or not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(src):
            cmd = ["g++", *flags, "-std=c++17", "-fPIC", "-shared", "-fopenmp", src, "-o", lib + ".tmp"]
            subprocess.check_call(cmd)
            os.replace(lib + ".tmp", lib)
    return LIB


_lib = None


class _Args(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int), ("num_elems", ctypes.c_int),
        ("coords", ctypes.c_void_p), ("tets", ctypes.c_void_p), ("elem_set", ctypes.c_void_p),
        ("mats", ctypes.c_void_p), ("model", ctypes.c_int), ("stabilization", ctypes.c_int),
        ("mode", ctypes.c_int), ("fad", ctypes.c_int), ("save", ctypes.c_int),
        ("qoi", ctypes.c_int), ("rho", ctypes.c_double), ("error_chain", ctypes.c_int),
        ("zu_diff", ctypes.c_void_p), ("zp_diff", ctypes.c_void_p), ("zp_coarse", ctypes.c_void_p),
        ("u", ctypes.c_void_p), ("p", ctypes.c_void_p),
        ("Fp_old", ctypes.c_void_p), ("eqps_old", ctypes.c_void_p), ("sigma_in", ctypes.c_void_p),
        ("sigma_out", ctypes.c_void_p), ("Fp_out", ctypes.c_void_p), ("eqps_out", ctypes.c_void_p),
        ("R", ctypes.c_void_p), ("row_ptr", ctypes.c_void_p), ("col_idx", ctypes.c_void_p),
        ("vals", ctypes.c_void_p), ("dMdu", ctypes.c_void_p), ("qoi_value", ctypes.c_void_p),
        ("num_plastic", ctypes.c_void_p), ("status", ctypes.c_void_p), ("fp_elastic_reset", ctypes.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_csr_graph.restype = ctypes.c_longlong
        L.orc_csr_graph.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]
        L.orc_assemble.restype = ctypes.c_int
        L.orc_assemble.argtypes = [ctypes.POINTER(_Args)]
        L.orc_assemble_parallel.restype = ctypes.c_int
        L.orc_assemble_parallel.argtypes = [ctypes.POINTER(_Args), ctypes.c_int]
        L.orc_apply_dbc.restype = None
        L.orc_apply_dbc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
        L.orc_apply_traction.restype = None
        L.orc_apply_traction.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
        L.orc_geometry.restype = None
        L.orc_geometry.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]
        L.orc_error.restype = ctypes.c_double
        L.orc_error.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_void_p]
        L.orc_expm.restype = None
        L.orc_expm.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------ graph
def csr_graph(num_nodes: int, tets: np.ndarray, neq: int = 4) -> Tuple[np.ndarray, np.ndarray]:
    L = lib()
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    nnz = L.orc_csr_graph(num_nodes, tets.shape[0], _p(tets), neq, None, None)
    row_ptr = np.zeros(num_nodes * neq + 1, np.int32)
    col_idx = np.zeros(nnz, np.int32)
    L.orc_csr_graph(num_nodes, tets.shape[0], _p(tets), neq, _p(row_ptr), _p(col_idx))
    return row_ptr, col_idx


def geometry(mesh):
    E = mesh.num_elems
    vol = np.zeros(E)
    h = np.zeros(E)
    grads = np.zeros((E, 4, 3))
    lib().orc_geometry(E, _p(mesh.coords), _p(mesh.tets), _p(vol), _p(h), _p(grads))
    return vol, h, grads


def expm(A: np.ndarray) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.float64).reshape(9)
    out = np.zeros(9)
    lib().orc_expm(_p(A), _p(out))
    return out.reshape(3, 3)


# ------------------------------------------------------------------ states
@dataclass
class States:
    """Per-element integration-point states (src/goal_states.cpp, goal_mechanics.cpp:87-95)."""
    sigma: np.ndarray
    Fp: np.ndarray
    Fp_old: np.ndarray
    eqps: np.ndarray
    eqps_old: np.ndarray

    @staticmethod
    def initial(num_elems: int) -> "States":
        I = np.tile(np.eye(3).ravel(), (num_elems, 1))
        return States(sigma=np.zeros((num_elems, 9)), Fp=I.copy(), Fp_old=I.copy(),
                      eqps=np.zeros(num_elems), eqps_old=np.zeros(num_elems))

    def update(self):
        """States::update: copy current -> _old (src/goal_states.cpp:130-141)."""
        self.Fp_old[:] = self.Fp
        self.eqps_old[:] = self.eqps

    def copy(self) -> "States":
        return States(*(a.copy() for a in (self.sigma, self.Fp, self.Fp_old, self.eqps, self.eqps_old)))


@dataclass
class Material:
    E: float
    nu: float
    K: float = 0.0
    Y: float = 0.0
    c0: float = 1.0

    def row(self):
        return [self.E, self.nu, self.K, self.Y, self.c0]


def assemble(mesh, model: int, mats: List[Material], u: np.ndarray, p: np.ndarray, states: States, *,
             mode: int, fad: bool, save: bool, stabilization: bool = True,
             qoi: int = QOI_NONE, rho: float = 0.0,
             graph: Optional[Tuple[np.ndarray, np.ndarray]] = None,
             R: Optional[np.ndarray] = None, vals: Optional[np.ndarray] = None, dMdu: Optional[np.ndarray] = None,
             error_weights: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None, threads: bool = False,
             fp_reset: bool = False):
    """One assemble(E, SolInfo*) of a chain; accumulates into R / vals / dMdu.
    ``fp_reset`` also writes Fp = Fp_old at elastic points (goal keeps the
    last plastic iterate's Fp there). Returns (qoi value, number of plastic
    points)."""
    L = lib()
    mats_arr = np.array([m.row() for m in mats], dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    a = _Args()
    a.num_nodes = mesh.num_nodes
    a.num_elems = mesh.num_elems
    a.coords = _p(mesh.coords)
    a.tets = _p(mesh.tets)
    es = np.ascontiguousarray(mesh.elem_set, dtype=np.int32)
    a.elem_set = _p(es)
    a.mats = _p(mats_arr)
    a.model = model
    a.stabilization = int(stabilization)
    a.mode = mode
    a.fad = int(fad)
    a.save = int(save)
    a.fp_elastic_reset = int(fp_reset)
    a.qoi = qoi
    a.rho = rho
    if error_weights is not None:
        zu, zp, zc = (np.ascontiguousarray(w, dtype=np.float64) for w in error_weights)
        a.error_chain = 1
        a.zu_diff, a.zp_diff, a.zp_coarse = _p(zu), _p(zp), _p(zc)
    a.u = _p(u)
    a.p = _p(p)
    a.Fp_old = _p(states.Fp_old)
    a.eqps_old = _p(states.eqps_old)
    a.sigma_in = _p(states.sigma)
    if save:
        a.sigma_out = _p(states.sigma)
        a.Fp_out = _p(states.Fp)
        a.eqps_out = _p(states.eqps)
    a.R = _p(R)
    if graph is not None:
        a.row_ptr = _p(graph[0])
        a.col_idx = _p(graph[1])
    a.vals = _p(vals)
    a.dMdu = _p(dMdu)
    q = np.zeros(1)
    npl = np.zeros(1, np.int32)
    st = np.zeros(1, np.int32)
    a.qoi_value = _p(q)
    a.num_plastic = _p(npl)
    a.status = _p(st)
    if threads:
        L.orc_assemble_parallel(ctypes.byref(a), 32768)
    else:
        L.orc_assemble(ctypes.byref(a))
    if st[0] != 0:
        raise RuntimeError("J2: return mapping failed")
    return float(q[0]), int(npl[0])


# ------------------------------------------------------------------ BCs
def eval_expr(expr: str, x: float, y: float, z: float, t: float) -> float:
    env = {k: getattr(math, k) for k in ("sin", "cos", "tan", "exp", "log", "sqrt", "pow", "fabs", "atan", "asin", "acos")}
    env["abs"] = abs
    env.update(x=x, y=y, z=z, t=t)
    return float(eval(expr.replace("^", "**"), {"__builtins__": {}}, env))


@dataclass
class DBC:
    eq: int
    node_set: str
    expr: str


@dataclass
class TBC:
    side_set: str
    exprs: Tuple[str, str, str]


def dbc_rows_values(mesh, dbcs: List[DBC], t: float):
    out = []
    for bc in dbcs:
        nodes = mesh.node_sets[bc.node_set]
        rows = (4 * nodes + bc.eq).astype(np.int32)
        vals = np.array([eval_expr(bc.expr, *mesh.coords[n], t) for n in nodes], dtype=np.float64)
        out.append((rows, vals))
    return out


def apply_dbcs(mesh, dbcs, t, u, R, graph=None, vals=None, dMdu=None, jac=False):
    L = lib()
    for rows, v in dbc_rows_values(mesh, dbcs, t):
        L.orc_apply_dbc(len(rows), _p(rows), _p(v), _p(np.ascontiguousarray(u)), int(jac), _p(R),
                        _p(graph[0]) if graph else None, _p(graph[1]) if graph else None, _p(vals), _p(dMdu))


def apply_tbcs(mesh, tbcs: List[TBC], t, R, zu: Optional[np.ndarray] = None):
    L = lib()
    for bc in tbcs:
        tris = np.ascontiguousarray(mesh.side_sets[bc.side_set], dtype=np.int32)
        xc = mesh.coords[tris].mean(axis=1)
        T = np.array([[eval_expr(e, *xc[s], t) for e in bc.exprs] for s in range(len(tris))],
                     dtype=np.float64).reshape(-1, 3)
        L.orc_apply_traction(len(tris), _p(tris), _p(mesh.coords), _p(T),
                             _p(np.ascontiguousarray(zu)) if zu is not None else None, _p(R))


# ------------------------------------------------------------------ solves
def csr_matrix(graph, vals, n):
    import scipy.sparse as sp
    return sp.csr_matrix((vals, graph[1], graph[0]), shape=(n, n))


@dataclass
class Problem:
    mesh: object
    model: int
    mats: List[Material]
    dbcs: List[DBC] = field(default_factory=list)
    tbcs: List[TBC] = field(default_factory=list)
    stabilization: bool = True
    qoi: int = QOI_AVG_DISP
    rho: float = 0.0
    fp_reset: bool = False   # Fp = Fp_old at elastic points (not goal's behaviour)


class Primal:
    """Newton solve of src/goal_primal.cpp:111-137 on the oracle."""

    def __init__(self, prob: Problem):
        self.prob = prob
        m = prob.mesh
        self.graph = csr_graph(m.num_nodes, m.tets)
        self.n = 4 * m.num_nodes
        self.u = np.zeros((m.num_nodes, 3))
        self.p = np.zeros(m.num_nodes)
        self.states = States.initial(m.num_elems)
        self.states.update()
        self.history: List[float] = []

    def compute_jacob(self, t_now, t_old):
        pr = self.prob
        R = np.zeros(self.n)
        vals = np.zeros(len(self.graph[1]))
        dMdu = np.zeros(self.n)
        assemble(pr.mesh, pr.model, pr.mats, self.u, self.p, self.states, mode=PRIMAL, fad=True, save=True,
                 stabilization=pr.stabilization, graph=self.graph, R=R, vals=vals, dMdu=dMdu, fp_reset=pr.fp_reset)
        apply_tbcs(pr.mesh, pr.tbcs, t_now, R)
        apply_dbcs(pr.mesh, pr.dbcs, t_now, self.u, R, self.graph, vals, dMdu, jac=True)
        return R, vals

    def compute_resid(self, t_now, t_old):
        pr = self.prob
        R = np.zeros(self.n)
        assemble(pr.mesh, pr.model, pr.mats, self.u, self.p, self.states, mode=PRIMAL, fad=False, save=True,
                 stabilization=pr.stabilization, R=R, fp_reset=pr.fp_reset)
        apply_tbcs(pr.mesh, pr.tbcs, t_now, R)
        apply_dbcs(pr.mesh, pr.dbcs, t_now, self.u, R)
        return R

    def solve(self, t_now, t_old, max_iters=5, tol=1e-8):
        import scipy.sparse.linalg as spla
        it = 1
        converged = False
        norms = []
        while it <= max_iters and not converged:
            R, vals = self.compute_jacob(t_now, t_old)
            R *= -1.0
            A = csr_matrix(self.graph, vals, self.n)
            du = spla.spsolve(A.tocsc(), R)
            self.u += du.reshape(-1, 4)[:, :3]
            self.p += du.reshape(-1, 4)[:, 3]
            R = self.compute_resid(t_now, t_old)
            norm = float(np.linalg.norm(R))
            norms.append(norm)
            if norm < tol:
                converged = True
            it += 1
        if not converged:
            raise RuntimeError(f"newton's method failed in {max_iters} iterations")
        self.history.append(len(norms))
        return norms

    def functional(self):
        pr = self.prob
        q, _ = assemble(pr.mesh, pr.model, pr.mats, self.u, self.p, self.states, mode=NONE, fad=False,
                        save=False, stabilization=pr.stabilization, qoi=pr.qoi, rho=pr.rho)
        return q


def run_primal(prob: Problem, num_steps: int, dt: float = 1.0, t0: float = 0.0, max_iters=5, tol=1e-8):
    """main_primal.cpp Solver::solve (src/main_primal.cpp:68-90)."""
    P = Primal(prob)
    t_old, t_now = t0, t0 + dt
    Js, its = [], []
    for _ in range(num_steps):
        norms = P.solve(t_now, t_old, max_iters, tol)
        its.append(len(norms))
        Js.append(P.functional())
        P.states.update()
        t_old, t_now = t_now, t_now + dt
    return P, Js, its


# ------------------------------------------------------------------ nested mesh
def edges_of(num_nodes: int, tets: np.ndarray) -> np.ndarray:
    """Unique mesh edges (i<j) ordered by (i, j): the upper triangle of the node graph."""
    t = tets
    pairs = np.concatenate([t[:, [a, b]] for a in range(4) for b in range(a + 1, 4)], axis=0).astype(np.int64)
    lo = pairs.min(axis=1)
    hi = pairs.max(axis=1)
    key = np.unique(lo * num_nodes + hi)
    return np.stack([key // num_nodes, key % num_nodes], axis=1).astype(np.int32)


_OCTA = [  # diagonal (a, b) and the cycle of the other four midpoints
    ((0, 5), (1, 2, 4, 3)),   # m01-m23 ; m02, m03, m13, m12
    ((1, 4), (0, 2, 5, 3)),   # m02-m13 ; m01, m03, m23, m12
    ((2, 3), (0, 1, 5, 4)),   # m03-m12 ; m01, m02, m23, m13
]
_MID = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def refine_uniform(mesh):
    """Declared uniform refinement rule shared by the oracle and the CUDA path:
    new node N+k at the midpoint of edge k (edges ordered as ``edges_of``);
    children of tet e are 8e..8e+7: the four corner tets, then the octahedron
    split along its shortest diagonal (first in m01-m23, m02-m13, m03-m12 order
    within a 1e-12 relative tie window), each child positively oriented.
    Returns (nested mesh, parent edges (Ne,2), child->parent element map)."""
    from goal_gb300.mesh import Mesh, orient_positive
    N = mesh.num_nodes
    E = mesh.num_elems
    edges = edges_of(N, mesh.tets)
    key = edges[:, 0].astype(np.int64) * N + edges[:, 1]
    coords = np.concatenate([mesh.coords, 0.5 * (mesh.coords[edges[:, 0]] + mesh.coords[edges[:, 1]])], axis=0)

    def mid(a, b):
        lo = np.minimum(a, b).astype(np.int64)
        hi = np.maximum(a, b).astype(np.int64)
        return (N + np.searchsorted(key, lo * N + hi)).astype(np.int32)

    t = mesh.tets
    m = np.stack([mid(t[:, a], t[:, b]) for a, b in _MID], axis=1)  # (E,6)
    v0, v1, v2, v3 = (t[:, k] for k in range(4))
    children = np.zeros((E, 8, 4), np.int32)
    children[:, 0] = np.stack([v0, m[:, 0], m[:, 1], m[:, 2]], 1)
    children[:, 1] = np.stack([m[:, 0], v1, m[:, 3], m[:, 4]], 1)
    children[:, 2] = np.stack([m[:, 1], m[:, 3], v2, m[:, 5]], 1)
    children[:, 3] = np.stack([m[:, 2], m[:, 4], m[:, 5], v3], 1)
    X = mesh.coords
    # diagonal lengths from parent coordinates: |x_c+x_d-x_a-x_b|^2
    d2 = np.zeros((E, 3))
    for k, ((i, j), _) in enumerate(_OCTA):
        a, b = _MID[i]
        c, d = _MID[j]
        vec = X[t[:, c]] + X[t[:, d]] - X[t[:, a]] - X[t[:, b]]
        d2[:, k] = vec[:, 0] * vec[:, 0] + vec[:, 1] * vec[:, 1] + vec[:, 2] * vec[:, 2]
    dmin = d2.min(axis=1)
    choice = np.where(d2[:, 0] <= dmin * (1 + 1e-12), 0, np.where(d2[:, 1] <= dmin * (1 + 1e-12), 1, 2))
    for k, ((i, j), cyc) in enumerate(_OCTA):
        sel = choice == k
        for c in range(4):
            children[sel, 4 + c] = np.stack([m[sel, i], m[sel, j], m[sel, cyc[c]], m[sel, cyc[(c + 1) % 4]]], 1)
    ctets = orient_positive(coords, children.reshape(-1, 4))
    parent = np.repeat(np.arange(E, dtype=np.int32), 8)
    node_sets = {}
    for name, nodes in mesh.node_sets.items():
        inset = np.zeros(N, bool)
        inset[nodes] = True
        extra = np.nonzero(inset[edges[:, 0]] & inset[edges[:, 1]])[0] + N
        node_sets[name] = np.concatenate([nodes, extra]).astype(np.int32)
    side_sets = {}
    for name, tris in mesh.side_sets.items():
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        mab, mbc, mca = mid(a, b), mid(b, c), mid(c, a)
        sub = np.stack([np.stack([a, mab, mca], 1), np.stack([mab, b, mbc], 1),
                        np.stack([mca, mbc, c], 1), np.stack([mab, mbc, mca], 1)], axis=1)
        side_sets[name] = np.ascontiguousarray(sub.reshape(-1, 3), dtype=np.int32)
    nested = Mesh(coords=np.ascontiguousarray(coords), tets=ctets, elem_set=np.repeat(mesh.elem_set, 8).astype(np.int32),
                  elem_set_names=list(mesh.elem_set_names), node_sets=node_sets, side_sets=side_sets)
    return nested, edges, parent


def prolong_nodal(values: np.ndarray, edges: np.ndarray) -> np.ndarray:
    """Edge-midpoint average onto the new nodes (Nested::set_coarse, src/goal_nested.cpp:369-393)."""
    return np.concatenate([values, 0.5 * (values[edges[:, 0]] + values[edges[:, 1]])], axis=0)


def nested_adjoint(primal: Primal, t_now: float, t_old: float):
    """NestedAdjoint::run on the uniformly refined mesh (src/goal_nested_adjoint.cpp:163-257).
    Returns dict with z, eta (= -R.z), bound, nested indicators, base indicators."""
    import scipy.sparse.linalg as spla
    pr = primal.prob
    nested, edges, parent = refine_uniform(pr.mesh)
    graph = csr_graph(nested.num_nodes, nested.tets)
    n = 4 * nested.num_nodes
    u = prolong_nodal(primal.u, edges)
    p = prolong_nodal(primal.p, edges)
    st = primal.states
    rep = lambda a: np.repeat(a, 8, axis=0)
    nst = States(sigma=rep(st.sigma), Fp=rep(st.Fp), Fp_old=rep(st.Fp_old), eqps=rep(st.eqps), eqps_old=rep(st.eqps_old))
    # compute_adjoint
    R = np.zeros(n)
    vals = np.zeros(len(graph[1]))
    dMdu = np.zeros(n)
    assemble(nested, pr.model, pr.mats, u, p, nst, mode=ADJOINT, fad=True, save=False,
             stabilization=pr.stabilization, qoi=pr.qoi, rho=pr.rho, graph=graph, R=R, vals=vals, dMdu=dMdu)
    apply_tbcs(nested, pr.tbcs, t_now, R)
    apply_dbcs(nested, pr.dbcs, t_now, u, R, graph, vals, dMdu, jac=True)
    A = csr_matrix(graph, vals, n)
    z = spla.spsolve(A.tocsc(), dMdu)
    eta = -float(R @ z)
    zf = z.reshape(-1, 4)
    N0 = pr.mesh.num_nodes
    zc = zf.copy()
    zc[N0:] = 0.5 * (zf[edges[:, 0]] + zf[edges[:, 1]])
    zd = zf - zc
    # localize (error chain)
    Re = np.zeros(n)
    assemble(nested, pr.model, pr.mats, u, p, nst, mode=PRIMAL, fad=False, save=False,
             stabilization=pr.stabilization, R=Re,
             error_weights=(np.ascontiguousarray(zd[:, :3]), np.ascontiguousarray(zd[:, 3]),
                            np.ascontiguousarray(zc[:, 3])))
    apply_tbcs(nested, pr.tbcs, t_now, Re, zu=np.ascontiguousarray(zd[:, :3]))
    apply_dbcs(nested, pr.dbcs, t_now, u, Re)
    ue = np.ascontiguousarray(Re.reshape(-1, 4)[:, :3])
    pe = np.ascontiguousarray(Re.reshape(-1, 4)[:, 3])
    elem_err = np.zeros(nested.num_elems)
    bound = lib().orc_error(nested.num_nodes, nested.num_elems, _p(nested.tets), _p(ue), _p(pe), _p(elem_err))
    base_err = np.zeros(pr.mesh.num_elems)
    np.add.at(base_err, parent, elem_err)
    return dict(nested=nested, graph=graph, A=A, R=R, dMdu=dMdu, z=z, eta=eta, bound=bound,
                elem_err=elem_err, base_err=base_err, z_coarse=zc, z_diff=zd, Re=Re, u=u, p=p,
                edges=edges, parent=parent)


# ------------------------------------------------------------------ tuned CPU baseline
class TunedAssembly:
    """The "tuned" CPU baseline of the primal Jacobian assembly (tuned.cpp):
    closed-form tangent, per-mesh geometry, coloured OpenMP scatter into 4x4
    blocks. A baseline timed beside the GPU path, checked against the
    dual-number restatement; not a checker itself."""

    def __init__(self, mesh, model: int, mats: List[Material], Fp_old: np.ndarray, stabilization: bool = True):
        build()
        L = ctypes.CDLL(TUNED_LIB)
        L.tuned_setup.restype = None
        L.tuned_setup.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 5
        L.tuned_color.restype = ctypes.c_int
        L.tuned_color.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.tuned_assemble.restype = ctypes.c_int
        L.tuned_assemble.argtypes = ([ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5 +
                                     [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_longlong] + [ctypes.c_void_p] * 5)
        self.L = L
        self.mesh = mesh
        self.model = model
        self.stab = int(stabilization)
        E, N = mesh.num_elems, mesh.num_nodes
        self.tets = np.ascontiguousarray(mesh.tets, dtype=np.int32)
        self.es = np.ascontiguousarray(mesh.elem_set, dtype=np.int32)
        self.mats = np.array([m.row() for m in mats], dtype=np.float64)
        self.Fp_old = np.ascontiguousarray(Fp_old, dtype=np.float64).reshape(E, 9)
        self.geo = np.zeros((E, 14))
        self.cpinv = np.zeros((E, 6))
        coords = np.ascontiguousarray(mesh.coords, dtype=np.float64)
        L.tuned_setup(E, _p(coords), _p(self.tets), _p(self.Fp_old), _p(self.geo), _p(self.cpinv))
        colors = np.zeros(E, np.int32)
        self.ncolors = L.tuned_color(N, E, _p(self.tets), _p(colors))
        if self.ncolors < 0:
            raise RuntimeError("tuned_color: more than 128 colours")
        self.order = np.ascontiguousarray(np.argsort(colors, kind="stable"), dtype=np.int32)
        self.color_ptr = np.ascontiguousarray(np.searchsorted(colors[self.order], np.arange(self.ncolors + 1)),
                                              dtype=np.int32)
        # node graph and the 16 block indices of every element
        a = np.repeat(self.tets, 4, axis=1).astype(np.int64)      # (E,16): node a of pair (a, b)
        b = np.tile(self.tets, (1, 4)).astype(np.int64)           # node b
        keys = a * N + b
        uniq = np.unique(keys)
        self.nnzb = len(uniq)
        rows = uniq // N
        self.brow_ptr = np.searchsorted(rows, np.arange(N + 1)).astype(np.int32)
        self.bcol = (uniq % N).astype(np.int32)
        self.blk = np.ascontiguousarray(np.searchsorted(uniq, keys), dtype=np.int32)
        self.R = np.zeros(4 * N)
        self.A = np.zeros(16 * self.nnzb)
        self.sigma = np.zeros((E, 9))
        self.Fp = self.Fp_old.copy()
        self.eqps = np.zeros(E)

    def assemble(self, U: np.ndarray, eqps_old: np.ndarray) -> int:
        """One primal Jacobian assembly with state writes; returns the return-map failures."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        eq = np.ascontiguousarray(eqps_old, dtype=np.float64)
        m = self.mesh
        return self.L.tuned_assemble(m.num_nodes, m.num_elems, _p(self.tets), _p(self.es), _p(self.mats), self.model,
                                     self.stab, _p(self.geo), _p(self.cpinv), _p(U), _p(self.Fp_old), _p(eq),
                                     self.ncolors, _p(self.color_ptr), _p(self.order), _p(self.blk), self.nnzb,
                                     _p(self.R), _p(self.A), _p(self.sigma), _p(self.Fp), _p(self.eqps))

    def csr_values(self) -> np.ndarray:
        """The blocks in the order of goal's scalar CSR graph (csr_graph)."""
        N = self.mesh.num_nodes
        deg = np.diff(self.brow_ptr)
        out = np.empty(16 * self.nnzb)
        Ab = self.A.reshape(-1, 4, 4)
        pos = 0
        for n in range(N):
            k0, k1 = self.brow_ptr[n], self.brow_ptr[n + 1]
            blk = Ab[k0:k1]                                       # (deg, 4, 4)
            rows = np.transpose(blk, (1, 0, 2)).reshape(4, -1)    # row r: blocks side by side
            out[pos:pos + rows.size] = rows.ravel()
            pos += rows.size
        assert pos == out.size and deg.sum() == self.nnzb
        return out
