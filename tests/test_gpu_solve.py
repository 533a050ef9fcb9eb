"""GPU linear solves, Newton and the nested adjoint / DWR estimate against the
oracle (calls through the C ABI).

* linear solve: true relative residual <= 1e-10 (the stopping rule), and the
  solution within 1e-8 relative of a direct solve of the oracle's matrix;
  FP64 and mixed (binary16-stored inner in FP32 arithmetic / FP64 outer)
  modes give the same answer.
* Newton on the reference's own 3D regression cases: the final QoI within the
  reference's tolerance (1e-8) of its stored value, and the same Newton
  iteration counts as the oracle.
* nested adjoint: eta = -R.z, the bound and the base-element indicators within
  1e-8 relative of the oracle (both solve to 1e-10; the oracle directly).
* a J2 load ramp on a 10^3 cube: Newton iteration counts and the QoI of every
  load step equal to the oracle's; the KS von Mises nested adjoint's eta from
  every GPU solver within 1e-8 relative of the oracle's direct solve.
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
@pytest.mark.parametrize("precision", [api.FP64, api.MIXED, api.MIXED_F32, api.NESTED_F64])
def test_linear_solve(model, mat, precision):
    d, m, s, A, b = _loaded_system(model, mat)
    x, st = api.solve(s, b, params=api.solve_params(krylov_size=100, max_iters=5000, tolerance=1e-10,
                                                   precision=precision, inner_iters=20))
    assert st["converged"]
    rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert rel <= 1.05e-10
    xd = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    if precision != api.FP64:
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
    onorms = P.solve(1.0, 0.0, max_iters=8, tol=1e-8)
    ref = O.nested_adjoint(P, 1.0, 0.0)
    # GPU primal + nested adjoint
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.NEOHOOKEAN, [mat.row()])
    s = api.SolInfo(d)
    bcs = api.Bcs(d, dbcs, tbcs)
    newton = api.primal_solve(m, s, bcs, 1.0, 0.0, 8, 1e-8, api.solve_params(tolerance=1e-12, max_iters=5000))
    assert newton["iters"] == len(onorms)  # the oracle's Newton iteration count
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


# ---------------------------------------------------------------- J2 ramp, 10^3
RAMP_INC, RAMP_STEPS = 0.0005, 3   # u_x = 0.0015 at the last step: the bar is plastic


def _ramp_oracle(mesh, inc=RAMP_INC, steps=RAMP_STEPS, fp_reset=False):
    mat = O.Material(200e3, 0.3, K=1000.0, Y=250.0, c0=1.0)
    dbcs = [O.DBC(0, "xmin", "0.0"), O.DBC(1, "xmin", "0.0"), O.DBC(2, "xmin", "0.0"),
            O.DBC(0, "xmax", f"{inc}*t")]
    P = O.Primal(O.Problem(mesh, O.J2, [mat], dbcs, [], qoi=O.QOI_KS, rho=20.0, fp_reset=fp_reset))
    its, Js = [], []
    for k in range(1, steps + 1):
        if k > 1:
            P.states.update()  # States::update after each converged step (src/main_nested.cpp:152)
        its.append(len(P.solve(float(k), float(k - 1), max_iters=15, tol=1e-8)))
        Js.append(P.functional())
    return P, its, Js, mat


@pytest.fixture(scope="module")
def j2_ramp():
    mesh = kuhn_cube(10, jitter=0.2, seed=1)
    P, its, Js, mat = _ramp_oracle(mesh)
    # the nested adjoint runs before the last step's States::update, as in
    # Solver::adapt inside the cycle loop (src/main_nested.cpp:128-153)
    ref = O.nested_adjoint(P, float(RAMP_STEPS), float(RAMP_STEPS - 1))
    return mesh, mat, its, Js, ref


def _ramp_gpu(mesh, mat, precision, inc=RAMP_INC, steps=RAMP_STEPS, fp_reset=False):
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.J2, [mat.row()], fp_reset=fp_reset)
    s = api.SolInfo(d)
    dbcs = [(0, "xmin", "0.0"), (1, "xmin", "0.0"), (2, "xmin", "0.0"), (0, "xmax", f"{inc}*t")]
    bcs = api.Bcs(d, dbcs, [])
    its, Js = [], []
    for k in range(1, steps + 1):
        if k > 1:
            m.update_states()
        r = api.primal_solve(m, s, bcs, float(k), float(k - 1), 15, 1e-8,
                             api.solve_params(tolerance=1e-10, precision=precision, inner_iters=30,
                                              krylov_size=30 if precision else 100, max_iters=5000))
        its.append(r["iters"])
        Js.append(api.assemble(m, None, api.NONE, jacobian=False, save_states=False, qoi=api.QOI_KS_VM, rho=20.0))
    return d, m, s, dbcs, its, Js


@pytest.mark.parametrize("precision", [api.FP64, api.MIXED])
def test_j2_ramp_newton_counts(j2_ramp, precision):
    """GPU Newton (FP64 or mixed linear solves) takes the oracle's Newton
    iteration count in every load step (src/goal_primal.cpp:111-137) and
    reaches the oracle's KS von Mises QoI after each step."""
    mesh, mat, oits, oJs, _ = j2_ramp
    _, _, _, _, its, Js = _ramp_gpu(mesh, mat, precision)
    assert its == oits
    for J, oJ in zip(Js, oJs):
        assert abs(J - oJ) <= 1e-10 * abs(oJ)


def test_j2_ramp_newton_counts_fp_reset():
    """The configuration's own increment (u_x += 0.002 per step) with the
    Fp_old reset option: 4 load steps, past the step where goal's state write
    makes Newton diverge; Newton counts and QoI of every step equal the
    oracle's with the same option, and the committed Fp equals the oracle's."""
    mesh = kuhn_cube(10, jitter=0.2, seed=1)
    P, oits, oJs, mat = _ramp_oracle(mesh, inc=0.002, steps=4, fp_reset=True)
    _, m, _, _, its, Js = _ramp_gpu(mesh, mat, api.MIXED, inc=0.002, steps=4, fp_reset=True)
    assert its == oits
    for J, oJ in zip(Js, oJs):
        assert abs(J - oJ) <= 1e-10 * abs(oJ)
    Fp = m.get_state(api.FP)
    assert np.abs(Fp - P.states.Fp).max() <= 1e-10


ADJOINT_ARMS = {
    "plain_fp64": dict(krylov_size=100, max_iters=30000),
    "nested_fp64": dict(krylov_size=30, max_iters=3000, precision=api.NESTED_F64, inner_iters=60),
    "mixed_f32": dict(krylov_size=30, max_iters=3000, precision=api.MIXED_F32, inner_iters=60),
    "mixed": dict(krylov_size=30, max_iters=3000, precision=api.MIXED, inner_iters=60),
    "learned_mixed": dict(krylov_size=30, max_iters=3000, precision=api.MIXED, inner_iters=60,
                          precond=api.PRECOND_LEARNED, learned_cap=1500),
}


@pytest.mark.parametrize("tol", [1e-10, 1e-12])
@pytest.mark.parametrize("arm", list(ADJOINT_ARMS))
def test_j2_nested_adjoint_eta(j2_ramp, arm, tol):
    """eta = -R.z of the KS von Mises nested adjoint after the J2 ramp, from
    every GPU solver arm, against the oracle's direct solve: within 1e-8
    relative, and the solve's true relative residual at its tolerance."""
    mesh, mat, _, _, ref = j2_ramp
    d, m, s, dbcs, _, _ = _ramp_gpu(mesh, mat, api.MIXED)
    na = api.NestedAdjoint(m, dbcs, [])
    prm = dict(ADJOINT_ARMS[arm])
    if prm.get("precond") == api.PRECOND_LEARNED:
        # training data the method produces: the last Newton Jacobian (with its
        # Dirichlet rows) and the nested adjoint's transposed Jacobian
        bcs = api.Bcs(d, dbcs, [])
        api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False)
        api.set_jac_dbcs(m, s, bcs, float(RAMP_STEPS))
        na.run(api.QOI_KS_VM, 20.0, float(RAMP_STEPS), float(RAMP_STEPS - 1), api.solve_params(max_iters=1))
        net = api.Learned(seed=0)
        net.train([s, na.si_handle()], epochs=60, lr=2e-3, num_probes=8)
        net.attach(na.si_handle())
    out = na.run(api.QOI_KS_VM, 20.0, float(RAMP_STEPS), float(RAMP_STEPS - 1),
                 api.solve_params(tolerance=tol, **prm))
    assert out["solve"]["converged"] and out["solve"]["rel_res"] <= tol
    assert not out["solve"]["fell_back"]
    dev = abs(out["eta"] - ref["eta"]) / abs(ref["eta"])
    print(f"{arm} tol {tol:g}: eta {out['eta']:.15e} oracle {ref['eta']:.15e} rel dev {dev:.2e} "
          f"iters {out['solve']['iters']}")
    assert dev <= 1e-8
    assert abs(out["bound"] - ref["bound"]) <= 1e-8 * abs(ref["bound"])
