"""Python mirror of goal's host interface on top of the C ABI.

Names follow the reference: ``Disc`` (src/goal_disc.hpp), ``Mechanics``
(src/goal_mechanics.hpp), ``SolInfo`` (src/goal_sol_info.hpp), ``assemble`` and
``EvalModes`` (src/goal_assembly.hpp, src/goal_eval_modes.hpp), the boundary
condition setters (src/goal_dbcs.hpp, src/goal_tbcs.hpp). Errors raise
``GoalError`` with the library's status and message (goal aborts instead).
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Optional, Sequence, Tuple

import numpy as np

from . import lib
from ._abi import Chain, DwrResult, NewtonStats, SolveParams, SolveStats

NONE, PRIMAL, ADJOINT = 0, 1, 2          # goal::EvalModes
NEOHOOKEAN, J2 = 0, 1
QOI_NONE, QOI_AVG_DISP, QOI_KS_VM = 0, 1, 2
SIGMA, FP, FP_OLD, EQPS, EQPS_OLD = 0, 1, 2, 3, 4
VEC_R, VEC_DMDU = 0, 1


class GoalError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[goal status {code}] {msg}")
        self.code = code


def check(rc: int):
    if rc != 0:
        msg = lib().goal_last_error()
        raise GoalError(rc, msg.decode() if isinstance(msg, bytes) else str(msg))


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class Disc:
    """Discretization on the GPU: mesh, DOF numbering, graph and colouring."""

    def __init__(self, mesh=None, _handle=None, _base=None):
        self._base = _base
        self.mesh = mesh
        L = lib()
        if _handle is not None:
            self.h = _handle
        else:
            h = ctypes.c_void_p()
            coords = _f64(mesh.coords)
            tets = _i32(mesh.tets)
            es = _i32(mesh.elem_set)
            check(L.goal_disc_create(mesh.num_nodes, mesh.num_elems, _ptr(coords), _ptr(tets), _ptr(es),
                                     max(1, len(mesh.elem_set_names)), ctypes.byref(h)))
            self.h = h
            for name, nodes in mesh.node_sets.items():
                n = _i32(nodes)
                check(L.goal_disc_add_node_set(self.h, name.encode(), len(n), _ptr(n)))
            for name, tris in mesh.side_sets.items():
                t = _i32(tris).reshape(-1, 3)
                check(L.goal_disc_add_side_set(self.h, name.encode(), t.shape[0], _ptr(t)))
            check(L.goal_disc_build_data(self.h))
        s = np.zeros(6, np.int64)
        check(L.goal_disc_sizes(self.h, _ptr(s)))
        self.num_nodes, self.num_elems, self.num_dofs, self.nnz, self.nnzb, self.num_colors = (int(x) for x in s)

    def graph(self) -> Tuple[np.ndarray, np.ndarray]:
        row_ptr = np.zeros(self.num_dofs + 1, np.int32)
        col_idx = np.zeros(self.nnz, np.int32)
        check(lib().goal_disc_get_graph(self.h, _ptr(row_ptr), _ptr(col_idx)))
        return row_ptr, col_idx

    def get_mesh(self):
        coords = np.zeros((self.num_nodes, 3))
        tets = np.zeros((self.num_elems, 4), np.int32)
        es = np.zeros(self.num_elems, np.int32)
        check(lib().goal_disc_get_mesh(self.h, _ptr(coords), _ptr(tets), _ptr(es)))
        return coords, tets, es

    def colors(self) -> np.ndarray:
        c = np.zeros(self.num_elems, np.int32)
        check(lib().goal_disc_get_colors(self.h, _ptr(c)))
        return c

    def stream(self) -> int:
        p = ctypes.c_void_p()
        check(lib().goal_disc_stream(self.h, ctypes.byref(p)))
        return int(p.value or 0)

    def build_times(self) -> dict:
        """Wall seconds of the build's phases and the colouring's round count."""
        t = np.zeros(5)
        rounds = ctypes.c_int()
        check(lib().goal_disc_build_times(self.h, _ptr(t), ctypes.byref(rounds)))
        return {"graph": float(t[0]), "colouring": float(t[1]), "layout": float(t[2]), "contribution_lists": float(t[3]),
                "sets": float(t[4]), "colour_rounds": int(rounds.value)}

    def nested(self) -> "Disc":
        """Nested(d, UNIFORM): uniformly refined copy."""
        h = ctypes.c_void_p()
        check(lib().goal_nested_create(self.h, ctypes.byref(h)))
        return Disc(_handle=h, _base=self)

    def parent_edges(self) -> np.ndarray:
        n = self.num_nodes - self._base.num_nodes
        e = np.zeros((n, 2), np.int32)
        check(lib().goal_nested_parent_edges(self.h, _ptr(e)))
        return e

    def close(self):
        if getattr(self, "h", None):
            lib().goal_disc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mechanics:
    """Model, materials, integration-point states and the nodal solution."""

    def __init__(self, disc: Disc, model: int, materials: Sequence[Sequence[float]], stabilization: bool = True,
                 fp_reset: bool = False):
        """``fp_reset``: J2 writes Fp = Fp_old at points that end elastic (goal
        keeps an earlier plastic Newton iterate's Fp there; see
        goal_mechanics_set_fp_reset)."""
        self.disc = disc
        self.model = model
        mats = _f64(materials).reshape(-1, 5)
        h = ctypes.c_void_p()
        check(lib().goal_mechanics_create(disc.h, model, _ptr(mats), int(stabilization), ctypes.byref(h)))
        self.h = h
        if fp_reset:
            check(lib().goal_mechanics_set_fp_reset(self.h, 1))

    def set_line_search(self, max_halvings: int):
        """Newton backtracking for goal_primal_solve (0: goal's full steps)."""
        check(lib().goal_mechanics_set_line_search(self.h, int(max_halvings)))

    def set_solution(self, U: np.ndarray):
        U = _f64(U).reshape(-1)
        assert U.size == self.disc.num_dofs
        check(lib().goal_mechanics_set_solution(self.h, _ptr(U)))

    def get_solution(self) -> np.ndarray:
        U = np.zeros(self.disc.num_dofs)
        check(lib().goal_mechanics_get_solution(self.h, _ptr(U)))
        return U

    def set_weights(self, z_diff: np.ndarray, z_coarse: np.ndarray):
        zd = _f64(z_diff).reshape(-1)
        zc = _f64(z_coarse).reshape(-1)
        check(lib().goal_mechanics_set_weights(self.h, _ptr(zd), _ptr(zc)))

    def get_state(self, which: int) -> np.ndarray:
        nc = 1 if which in (EQPS, EQPS_OLD) else 9
        out = np.zeros(self.disc.num_elems * nc)
        check(lib().goal_states_get(self.h, which, _ptr(out)))
        return out if nc == 1 else out.reshape(-1, 9)

    def set_state(self, which: int, values: np.ndarray):
        v = _f64(values).reshape(-1)
        check(lib().goal_states_set(self.h, which, _ptr(v)))

    def update_states(self):
        check(lib().goal_states_update(self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().goal_mechanics_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SolInfo:
    """R, dMdu and dRdu (4x4-block storage) of one discretization."""

    def __init__(self, disc: Disc):
        self.disc = disc
        h = ctypes.c_void_p()
        check(lib().goal_sol_info_create(disc.h, ctypes.byref(h)))
        self.h = h

    def zero_all(self):
        check(lib().goal_sol_info_zero_all(self.h))

    def vector(self, which: int) -> np.ndarray:
        out = np.zeros(self.disc.num_dofs)
        check(lib().goal_sol_info_get_vector(self.h, which, _ptr(out)))
        return out

    def set_vector(self, which: int, values: np.ndarray):
        v = _f64(values).reshape(-1)
        check(lib().goal_sol_info_set_vector(self.h, which, _ptr(v)))

    @property
    def R(self) -> np.ndarray:
        return self.vector(VEC_R)

    @property
    def dMdu(self) -> np.ndarray:
        return self.vector(VEC_DMDU)

    def dRdu_csr(self) -> np.ndarray:
        out = np.zeros(self.disc.nnz)
        check(lib().goal_sol_info_get_dRdu_csr(self.h, _ptr(out)))
        return out

    def dRdu_bsr(self) -> np.ndarray:
        out = np.zeros(16 * self.disc.nnzb)
        check(lib().goal_sol_info_get_dRdu_bsr(self.h, _ptr(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().goal_sol_info_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assemble(mech: Mechanics, sol_info: Optional[SolInfo], mode: int, jacobian: bool, save_states: bool,
             qoi: int = QOI_NONE, rho: float = 0.0, error_chain: bool = False, overwrite: bool = True,
             colored: bool = False) -> float:
    """assemble(E, SolInfo*) for one evaluator chain; returns the QoI value."""
    c = Chain(mode=mode, jacobian=int(jacobian), save_states=int(save_states), qoi=qoi, rho=rho,
              error_chain=int(error_chain), overwrite=int(overwrite), colored=int(colored))
    q = ctypes.c_double(0.0)
    check(lib().goal_assemble(mech.h, sol_info.h if sol_info is not None else None, ctypes.byref(c), ctypes.byref(q)))
    return q.value


class Bcs:
    """Dirichlet [eq, node set, expr] and traction [side set, Tx, Ty, Tz] conditions."""

    def __init__(self, disc: Disc, dirichlet: Iterable = (), traction: Iterable = ()):
        self.disc = disc
        h = ctypes.c_void_p()
        check(lib().goal_bcs_create(disc.h, ctypes.byref(h)))
        self.h = h
        for eq, ns, expr in dirichlet:
            check(lib().goal_bcs_add_dirichlet(self.h, int(eq), ns.encode(), expr.encode()))
        for ss, tx, ty, tz in traction:
            check(lib().goal_bcs_add_traction(self.h, ss.encode(), tx.encode(), ty.encode(), tz.encode()))

    def close(self):
        if getattr(self, "h", None):
            lib().goal_bcs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_resid_dbcs(mech: Mechanics, s: SolInfo, bcs: Bcs, t: float):
    check(lib().goal_set_resid_dbcs(mech.h, s.h, bcs.h, t))


def set_jac_dbcs(mech: Mechanics, s: SolInfo, bcs: Bcs, t: float):
    check(lib().goal_set_jac_dbcs(mech.h, s.h, bcs.h, t))


def set_tbcs(mech: Mechanics, s: SolInfo, bcs: Bcs, t: float, error_weights: bool = False):
    check(lib().goal_set_tbcs(mech.h, s.h, bcs.h, t, int(error_weights)))


def eval_expr(expr: str, x: float, y: float, z: float, t: float) -> float:
    out = ctypes.c_double()
    check(lib().goal_eval(expr.encode(), x, y, z, t, ctypes.byref(out)))
    return out.value


FP64, MIXED, MIXED_F32, NESTED_F64 = 0, 1, 2, 3  # precision: FP64; inner solve in binary16 / FP32 / FP64
PRECOND_BJ, PRECOND_LEARNED = 0, 1


def solve_params(krylov_size=100, max_iters=2000, tolerance=1e-10, precision=FP64, inner_iters=30,
                 precond=PRECOND_BJ, learned_cap=0) -> SolveParams:
    return SolveParams(krylov_size=krylov_size, max_iters=max_iters, tolerance=tolerance, precision=precision,
                       inner_iters=inner_iters, precond=precond, learned_cap=learned_cap)


def _stats_dict(st: SolveStats) -> dict:
    return dict(iters=st.iters, inner_iters=st.inner_iters, converged=bool(st.converged), fell_back=bool(st.fell_back),
                rel_res=st.rel_res, seconds=st.seconds, spmv64=st.spmv64, spmv32=st.spmv32)


def solve(sol_info: SolInfo, b: np.ndarray, x0: Optional[np.ndarray] = None, params: Optional[SolveParams] = None):
    """goal::solve on dRdu of the SolInfo; returns (x, stats)."""
    b = _f64(b).reshape(-1)
    x = np.zeros_like(b) if x0 is None else _f64(x0).reshape(-1).copy()
    st = SolveStats()
    check(lib().goal_solve(sol_info.h, ctypes.byref(params or solve_params()), _ptr(b), _ptr(x), ctypes.byref(st)))
    return x, _stats_dict(st)


def primal_solve(mech: Mechanics, s: SolInfo, bcs: Bcs, t_now: float, t_old: float, max_iters: int = 5,
                 tolerance: float = 1e-8, params: Optional[SolveParams] = None) -> dict:
    """Primal::solve (Newton); raises GoalError(GOAL_ERR_NEWTON) when it fails."""
    st = NewtonStats()
    rc = lib().goal_primal_solve(mech.h, s.h, bcs.h, t_now, t_old, max_iters, tolerance,
                                 ctypes.byref(params or solve_params()), ctypes.byref(st))
    out = dict(iters=st.iters, converged=bool(st.converged), linear_iters=st.linear_iters,
               inner_iters=st.inner_iters, norms=list(st.norms[:min(st.iters, 32)]),
               seconds_assembly=st.seconds_assembly, seconds_solve=st.seconds_solve, backtracks=st.backtracks)
    if rc != 0:
        try:
            check(rc)
        except GoalError as e:
            e.stats = out
            raise
    return out


class NestedAdjoint:
    """NestedAdjoint: adjoint on the uniformly refined mesh and the DWR estimate."""

    def __init__(self, base_mech: Mechanics, dirichlet=(), traction=()):
        h = ctypes.c_void_p()
        check(lib().goal_nested_adjoint_create(base_mech.h, ctypes.byref(h)))
        self.h = h
        self.base = base_mech
        dh = ctypes.c_void_p()
        check(lib().goal_nested_adjoint_disc(self.h, ctypes.byref(dh)))
        self.disc = Disc.__new__(Disc)
        self.disc._base = base_mech.disc
        self.disc.mesh = None
        self.disc.h = dh
        sizes = np.zeros(6, np.int64)
        check(lib().goal_disc_sizes(dh, _ptr(sizes)))
        (self.disc.num_nodes, self.disc.num_elems, self.disc.num_dofs, self.disc.nnz, self.disc.nnzb,
         self.disc.num_colors) = (int(x) for x in sizes)
        self.bcs = Bcs(self.disc, dirichlet, traction)

    def run(self, qoi: int, rho: float, t_now: float, t_old: float, params: Optional[SolveParams] = None,
            nested_error: bool = False) -> dict:
        r = DwrResult()
        be = np.zeros(self.base.disc.num_elems)
        ne = np.zeros(self.disc.num_elems) if nested_error else None
        check(lib().goal_nested_adjoint_run(self.h, self.bcs.h, qoi, rho, t_now, t_old,
                                            ctypes.byref(params or solve_params()), ctypes.byref(r), _ptr(be),
                                            _ptr(ne)))
        out = dict(eta=r.eta, bound=r.bound, qoi=r.qoi, solve=_stats_dict(r.solve), base_error=be,
                   seconds_adjoint=r.seconds_adjoint, seconds_solve=r.seconds_solve,
                   seconds_localize=r.seconds_localize)
        if ne is not None:
            out["nested_error"] = ne
        return out

    def si_handle(self) -> "SolInfo":
        """The nested linear objects (a non-owning SolInfo view)."""
        sh = ctypes.c_void_p()
        check(lib().goal_nested_adjoint_sol_info(self.h, ctypes.byref(sh)))
        view = SolInfo.__new__(SolInfo)
        view.disc = self.disc
        view.h = sh
        view.close = lambda: None
        return view

    def z(self) -> np.ndarray:
        z = np.zeros(self.disc.num_dofs)
        check(lib().goal_nested_adjoint_get_z(self.h, _ptr(z)))
        return z

    def close(self):
        if getattr(self, "h", None):
            self.bcs.close()
            self.disc.h = None  # owned by the nested adjoint
            lib().goal_nested_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Learned:
    """The learned block-Jacobi correction (mesh-graph network, see goal_gb300.h)."""

    def __init__(self, seed: int = 0):
        h = ctypes.c_void_p()
        check(lib().goal_learned_create(seed, ctypes.byref(h)))
        self.h = h
        n = ctypes.c_int()
        check(lib().goal_learned_num_params(self.h, ctypes.byref(n)))
        self.num_params = n.value

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(lib().goal_learned_get_params(self.h, _ptr(out)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().goal_learned_set_params(self.h, _ptr(p)))

    def loss_grad(self, s: SolInfo, probes: Optional[np.ndarray] = None, num_probes: int = 4, seed: int = 0):
        loss = ctypes.c_double()
        grad = np.zeros(self.num_params, np.float32)
        if probes is not None:
            pr = np.ascontiguousarray(probes, dtype=np.float64)
            num_probes = pr.shape[0]
        else:
            pr = None
        check(lib().goal_learned_loss_grad(self.h, s.h, num_probes, _ptr(pr), seed, ctypes.byref(loss), _ptr(grad)))
        return loss.value, grad

    def corrections(self, s: SolInfo) -> np.ndarray:
        C = np.zeros((s.disc.num_nodes, 16), np.float32)
        check(lib().goal_learned_corrections(self.h, s.h, _ptr(C)))
        return C

    def train(self, systems, epochs: int = 50, lr: float = 1e-3, num_probes: int = 8, seed: int = 0) -> np.ndarray:
        arr = (ctypes.c_void_p * len(systems))(*[x.h.value for x in systems])
        losses = np.zeros(epochs)
        check(lib().goal_learned_train(self.h, arr, len(systems), epochs, lr, num_probes, seed, _ptr(losses)))
        return losses

    def attach(self, s: SolInfo):
        check(lib().goal_sol_info_set_learned(s.h, self.h))

    def close(self):
        if getattr(self, "h", None):
            lib().goal_learned_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def size_field(disc: Disc, elem_error, target: int) -> np.ndarray:
    """get_iso_target_size (src/goal_size_field.cpp:139-151): per-node target
    sizes from per-element error indicators and a target element count."""
    err = _f64(elem_error)
    if err.shape != (disc.num_elems,):
        raise ValueError("one error indicator per element")
    out = np.zeros(disc.num_nodes)
    check(lib().goal_size_field(disc.h, _ptr(err), int(target), _ptr(out)))
    return out
