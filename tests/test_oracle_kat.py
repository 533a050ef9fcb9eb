"""Pins the oracle against the reference's own regression values.

The reference's examples run GoalPrimal on test/mesh/cube and assert the final
QoI (src/goal_regression.cpp:14-23). The oracle must reproduce each value
within the example's own tolerance (1e-8 absolute); in practice it agrees to
~1e-16, i.e. the element chain, the J2 history, the BCs and the QoI are
restated exactly.
"""
import numpy as np
import pytest

from oracle import oracle as O

MODEL = {"neohookean": O.NEOHOOKEAN, "J2": O.J2}


def problem_from_case(mesh, c):
    mats = [O.Material(c["E"], c["nu"], K=c["K"], Y=c["Y"], c0=c["c0"])]
    dbcs = [O.DBC(int(eq), s, e) for eq, s, e in c["dirichlet"]]
    tbcs = [O.TBC(t[0], tuple(t[1:])) for t in c["traction"]]
    return O.Problem(mesh, MODEL[c["model"]], mats, dbcs, tbcs, qoi=O.QOI_AVG_DISP)


@pytest.mark.parametrize("case", ["neohookean_uniaxial_3D", "J2_uniaxial_3D", "J2_traction_3D"])
def test_regression_value(cube_kat, case):
    mesh, cases = cube_kat
    c = cases[case]
    prob = problem_from_case(mesh, c)
    P, Js, its = O.run_primal(prob, c["num_steps"], c["step_size"], 0.0, c["newton_max_iters"], c["newton_tol"])
    assert abs(Js[-1] - c["value"]) < c["tolerance"]
    # much tighter than the reference's own check: the restatement is exact
    assert abs(Js[-1] - c["value"]) < 1e-14


def test_expression_kat():
    """test/control.cpp:12-15: sin(x)*cos(y) + 2*exp(t) - z at (1,2,3,4)."""
    import math
    v1 = O.eval_expr("sin(x)*cos(y) + 2*exp(t) - z", 1.0, 2.0, 3.0, 4.0)
    v2 = math.sin(1.0) * math.cos(2.0) + 2.0 * math.exp(4.0) - 3.0
    assert abs(v1 - v2) < 1e-15


def test_mesh_fixture(cube_kat):
    mesh, _ = cube_kat
    assert mesh.num_nodes == 51 and mesh.num_elems == 132
    assert abs(mesh.volumes().sum() - 1.0) < 1e-12
    assert (mesh.volumes() > 0).all()
    for name in ("xmin", "xmax", "ymin", "zmin", "zmax"):
        assert len(mesh.node_sets[name]) == 13


def test_jacobian_matches_finite_differences(cube_kat):
    """The dual-number Jacobian of the oracle vs central differences of its residual."""
    mesh, cases = cube_kat
    for model, mat in ((O.NEOHOOKEAN, O.Material(1000.0, 0.25, c0=1.0)),
                       (O.J2, O.Material(1000.0, 0.25, K=100.0, Y=10.0, c0=1.0))):
        rng = np.random.default_rng(1)
        u = 0.02 * rng.standard_normal((mesh.num_nodes, 3))
        p = 5.0 * rng.standard_normal(mesh.num_nodes)
        st = O.States.initial(mesh.num_elems)
        g = O.csr_graph(mesh.num_nodes, mesh.tets)
        n = 4 * mesh.num_nodes
        R = np.zeros(n); vals = np.zeros(len(g[1]))
        O.assemble(mesh, model, [mat], u, p, st, mode=O.PRIMAL, fad=True, save=False, graph=g, R=R, vals=vals)
        A = O.csr_matrix(g, vals, n).toarray()
        eps = 1e-6
        for col in (0, 5, 7, 42, 103):
            up, pp = u.copy(), p.copy()
            um, pm = u.copy(), p.copy()
            node, eq = divmod(col, 4)
            if eq < 3:
                up[node, eq] += eps; um[node, eq] -= eps
            else:
                pp[node] += eps; pm[node] -= eps
            Rp = np.zeros(n); Rm = np.zeros(n)
            O.assemble(mesh, model, [mat], up, pp, st, mode=O.PRIMAL, fad=False, save=False, R=Rp)
            O.assemble(mesh, model, [mat], um, pm, st, mode=O.PRIMAL, fad=False, save=False, R=Rm)
            fd = (Rp - Rm) / (2 * eps)
            scale = np.abs(A[:, col]).max()
            assert np.abs(fd - A[:, col]).max() < 1e-6 * scale
