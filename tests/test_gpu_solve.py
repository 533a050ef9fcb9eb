"""GPU linear solves, Newton and the nested adjoint / DWR estimate against the
oracle (calls through the C ABI).

* linear solve: true relative residual <= 1e-10 (the stopping rule), and the
  solution within 1e-8 relative of a direct solve of the oracle's matrix;
  FP64 and mixed (FP32 inner / FP64 outer) modes give the same answer.
* Newton on the reference's own 3D regression cases: the final QoI within the
  reference's tolerance (1e-8) of its stored value, and the same Newton
  iteration counts as the oracle.
* nested adjoint: eta = -R.z, the bound and the base-element indicators within
  1e-8 relative of the oracle (both solve to 1e-10; the oracle directly).
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import oracle as O
from goal_gb300 import api
from goal_gb300.mesh import kuhn_cube

pytestmark = pytest.mark.gpu

MODEL = {"neohookean": O.NEOHOOKEAN, "J2": O.J2}


def _loaded_system(model, mat, n=6):
    """Jacobian (with Dirichlet rows) at the converged state of one load step of
    a stretched Kuhn cube, and the adjoint right-hand side dM/du of avg disp."""
    mesh = kuhn_cube(n)
    d = api.Disc(mesh)
    m = api.Mechanics(d, model, [mat.row()])
    s = api.SolInfo(d)
    bcs = api.Bcs(d, [(0, "xmin", "0.0"), (1, "ymin", "0.0"), (2, "zmin", "0.0"), (0, "xmax", "0.002*t")], [])
    api.primal_solve(m, s, bcs, 1.0, 0.0, 8, 1e-8, api.solve_params(tolerance=1e-10, precision=api.MIXED))
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, qoi=api.QOI_AVG_DISP)
    api.set_jac_dbcs(m, s, bcs, 1.0)
    g = d.graph()
    A = O.csr_matrix(g, s.dRdu_csr(), d.num_dofs)
    return d, m, s, A, s.dMdu


MATS = [(O.NEOHOOKEAN, O.Material(1000.0, 0.25, c0=1.0)), (O.J2, O.Material(200e3, 0.3, K=1000.0, Y=250.0, c0=1.0)),
        # nearly incompressible (the Cook's membrane example's nu): the pressure
        # block is tiny next to the displacement block; the mixed solver's
        # dof-scaled binary16 inner matrix must still hold it
        (O.NEOHOOKEAN, O.Material(1000.0, 0.4999, c0=1.0))]


@pytest.mark.parametrize("model,mat", MATS)
@pytest.mark.parametrize("precision", [api.FP64, api.MIXED])
def test_linear_solve(model, mat, precision):
    d, m, s, A, b = _loaded_system(model, mat)
    x, st = api.solve(s, b, params=api.solve_params(krylov_size=100, max_iters=5000, tolerance=1e-10,
                                                   precision=precision, inner_iters=20))
    assert st["converged"]
    rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert rel <= 1.05e-10
    xd = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    if precision == api.MIXED:
        assert st["inner_iters"] > 0 and st["spmv32"] > 0


def test_mixed_needs_fewer_outer_iterations():
    d, m, s, A, b = _loaded_system(*MATS[1])  # J2
    _, s64 = api.solve(s, b, params=api.solve_params(tolerance=1e-10, max_iters=5000))
    _, smx = api.solve(s, b, params=api.solve_params(tolerance=1e-10, max_iters=5000, precision=api.MIXED,
                                                     inner_iters=30))
    assert s64["converged"] and smx["converged"]
    assert smx["iters"] < s64["iters"]
    # the mixed solve is bitwise repeatable
    x1, s1 = api.solve(s, b, params=api.solve_params(tolerance=1e-10, max_iters=5000, precision=api.MIXED,
                                                     inner_iters=30))
    x2, s2 = api.solve(s, b, params=api.solve_params(tolerance=1e-10, max_iters=5000, precision=api.MIXED,
                                                     inner_iters=30))
    assert np.array_equal(x1, x2) and s1["iters"] == s2["iters"]


@pytest.mark.parametrize("case", ["neohookean_uniaxial_3D", "J2_uniaxial_3D", "J2_traction_3D"])
@pytest.mark.parametrize("precision", [api.FP64, api.MIXED])
def test_newton_regression_values(cube_kat, case, precision):
    mesh, cases = cube_kat
    c = cases[case]
    d = api.Disc(mesh)
    m = api.Mechanics(d, MODEL[c["model"]], [[c["E"], c["nu"], c["K"], c["Y"], c["c0"]]])
    s = api.SolInfo(d)
    bcs = api.Bcs(d, [(int(a), b_, e) for a, b_, e in c["dirichlet"]], [tuple(t) for t in c["traction"]])
    t_old, t_now = 0.0, c["step_size"]
    its = []
    for _ in range(c["num_steps"]):
        r = api.primal_solve(m, s, bcs, t_now, t_old, c["newton_max_iters"], c["newton_tol"],
                             api.solve_params(tolerance=1e-10, precision=precision, inner_iters=20))
        its.append(r["iters"])
        J = api.assemble(m, None, api.NONE, jacobian=False, save_states=False, qoi=api.QOI_AVG_DISP)
        m.update_states()
        t_old, t_now = t_now, t_now + c["step_size"]
    assert abs(J - c["value"]) < c["tolerance"]
    # Newton iteration counts of the oracle (direct linear solves)
    from tests.test_oracle_kat import problem_from_case
    _, Js, oits = O.run_primal(problem_from_case(mesh, c), c["num_steps"], c["step_size"], 0.0,
                               c["newton_max_iters"], c["newton_tol"])
    assert its == oits
    assert abs(J - Js[-1]) <= 1e-10 * abs(Js[-1])


def _primal_problem(n=4):
    mesh = kuhn_cube(n)
    mat = O.Material(1000.0, 0.25, c0=1.0)
    dbcs = [(0, "xmin", "0.0"), (1, "xmin", "0.0"), (2, "xmin", "0.0")]
    tbcs = [("xmax", "10.0*t", "0.0", "0.0")]
    return mesh, mat, dbcs, tbcs


@pytest.mark.parametrize("n,qoi", [(4, api.QOI_AVG_DISP), (4, api.QOI_KS_VM),
                                   # the small published-size case: 10^3 cube, neo-Hookean, traction
                                   # (10, 0, 0) on x=1, avg disp, nested mesh of 48,000 tets
                                   (10, api.QOI_AVG_DISP)])
def test_nested_adjoint_matches_oracle(n, qoi):
    mesh, mat, dbcs, tbcs = _primal_problem(n)
    rho = 20.0
    # oracle primal + nested adjoint
    prob = O.Problem(mesh, O.NEOHOOKEAN, [mat], [O.DBC(*b) for b in dbcs],
                     [O.TBC(t[0], tuple(t[1:])) for t in tbcs], qoi=qoi, rho=rho)
    P = O.Primal(prob)
    P.solve(1.0, 0.0, max_iters=8, tol=1e-8)
    ref = O.nested_adjoint(P, 1.0, 0.0)
    # GPU primal + nested adjoint
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.NEOHOOKEAN, [mat.row()])
    s = api.SolInfo(d)
    bcs = api.Bcs(d, dbcs, tbcs)
    api.primal_solve(m, s, bcs, 1.0, 0.0, 8, 1e-8, api.solve_params(tolerance=1e-12, max_iters=5000))
    na = api.NestedAdjoint(m, dbcs, tbcs)
    out = na.run(qoi, rho, 1.0, 0.0, api.solve_params(tolerance=1e-12, max_iters=20000), nested_error=True)
    if n == 10:
        assert na.disc.num_elems == 48000
    assert out["solve"]["converged"]
    assert abs(out["eta"] - ref["eta"]) <= 1e-8 * abs(ref["eta"])
    assert abs(out["bound"] - ref["bound"]) <= 1e-8 * abs(ref["bound"])
    be = out["base_error"]
    assert np.abs(be - ref["base_err"]).max() <= 1e-8 * np.abs(ref["base_err"]).max()
    z = na.z()
    assert np.linalg.norm(z - ref["z"]) <= 1e-8 * np.linalg.norm(ref["z"])
