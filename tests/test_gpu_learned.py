"""The learned block-Jacobi correction on the GPU.

* forward outputs and the loss gradient of the CUDA kernels against the numpy
  restatement (oracle/mpnn.py) on the same weights and probes (float32
  arithmetic, summation order differs: 1e-4 relative);
* training on Jacobians the method produces (Newton systems of a J2 load step)
  lowers the loss;
* on a held-out system (another mesh) the trained network needs fewer FGMRES
  iterations than plain block-Jacobi, the method without it (the gain is
  printed), converges to the same 1e-10 relative residual and solution, and
  the iteration cap falls back to plain block-Jacobi.

The meshes are Kuhn cubes with jittered interior nodes: on the exact grid the
matrix inherits the grid's translation symmetry (repeated eigenvalues), which
no mesh of a real part has.
"""
import numpy as np
import pytest

from oracle import mpnn as M
from goal_gb300 import api
from goal_gb300.mesh import kuhn_cube

pytestmark = pytest.mark.gpu

MAT = [200e3, 0.3, 1000.0, 250.0, 1.0]


def bsr_host(d, s):
    rp, ci = d.graph()
    N = d.num_nodes
    A = s.dRdu_bsr().reshape(-1, 4, 4)
    deg = (rp[1:4 * N + 1:4] - rp[0:4 * N:4]) // 4
    brow = np.concatenate([[0], np.cumsum(deg)])
    bcol = np.concatenate([ci[rp[4 * n]:rp[4 * n] + 4 * deg[n]:4] // 4 for n in range(N)])
    diag = np.array([brow[n] + np.searchsorted(bcol[brow[n]:brow[n + 1]], n) for n in range(N)])
    return brow, bcol, diag, A


def newton_system(n, steps, seed=0):
    """The Newton system after ``steps`` J2 load steps (u_x = 0.001 t on x=1)."""
    mesh = kuhn_cube(n, jitter=0.2, seed=seed)
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.J2, [MAT])
    s = api.SolInfo(d)
    bcs = api.Bcs(d, [(0, "xmin", "0.0"), (1, "xmin", "0.0"), (2, "xmin", "0.0"), (0, "xmax", "0.001*t")], [])
    for k in range(1, steps + 1):
        if k > 1:
            m.update_states()
        api.primal_solve(m, s, bcs, float(k), float(k - 1), 15, 1e-8,
                         api.solve_params(tolerance=1e-10, precision=api.MIXED))
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, qoi=api.QOI_AVG_DISP)
    api.set_jac_dbcs(m, s, bcs, float(steps))
    return d, m, s, bcs


def test_forward_and_gradient_match_restatement():
    mesh = kuhn_cube(3)
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.J2, [MAT])
    s = api.SolInfo(d)
    rng = np.random.default_rng(0)
    U = np.zeros((mesh.num_nodes, 4))
    U[:, :3] = 1e-3 * rng.standard_normal((mesh.num_nodes, 3))
    U[:, 3] = rng.standard_normal(mesh.num_nodes)
    m.set_solution(U.ravel())
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False)
    brow, bcol, diag, A = bsr_host(d, s)
    net = api.Learned(seed=3)
    theta = net.params() + 0.02 * rng.standard_normal(net.num_params).astype(np.float32)
    net.set_params(theta)
    probes = rng.standard_normal((3, d.num_dofs))
    lg, gg = net.loss_grad(s, probes=probes)
    lo, go = M.loss_and_grad(theta, brow, bcol, diag, A, list(probes))
    assert abs(lg - lo) <= 1e-6 * abs(lo)
    assert np.linalg.norm(gg - go) <= 1e-4 * np.linalg.norm(go)
    x, e, sd, Di, dirichlet = M.features(brow, bcol, diag, A)
    Co = M.forward(M.unflatten(theta), brow, bcol, diag, x, e)
    C = net.corrections(s)
    assert np.abs(C - Co).max() <= 1e-4 * np.abs(Co).max()


def test_training_and_gain_over_block_jacobi():
    systems = [newton_system(8, k, seed=k) for k in (1, 2, 3)]
    net = api.Learned(seed=0)
    losses = net.train([x[2] for x in systems], epochs=60, lr=2e-3, num_probes=8)
    assert losses[-1] < 0.5 * losses[0]
    d, m, s, bcs = newton_system(10, 2, seed=99)  # held out: another mesh
    b = s.dMdu
    prm = dict(tolerance=1e-10, max_iters=20000, krylov_size=100)
    x0, plain = api.solve(s, b, params=api.solve_params(**prm))
    net.attach(s)
    x1, learned = api.solve(s, b, params=api.solve_params(precond=api.PRECOND_LEARNED, **prm))
    print(f"\nFGMRES iterations to 1e-10: plain block-Jacobi {plain['iters']}, learned {learned['iters']}")
    assert plain["converged"] and learned["converged"]
    assert learned["iters"] < 0.8 * plain["iters"]
    assert np.linalg.norm(x1 - x0) <= 1e-7 * np.linalg.norm(x0)
    # the learned two-sweep inside the binary16-inner / FP64-outer solve: the same
    # solution, fewer outer iterations than plain block-Jacobi in that solver,
    # and bitwise repeatable (fixed reduction orders, no atomics)
    pm = dict(prm, krylov_size=30, precision=api.MIXED, inner_iters=30)
    x3, lm = api.solve(s, b, params=api.solve_params(precond=api.PRECOND_LEARNED, **pm))
    x4, lm2 = api.solve(s, b, params=api.solve_params(precond=api.PRECOND_LEARNED, **pm))
    assert lm["converged"] and not lm["fell_back"]
    assert np.array_equal(x3, x4) and lm["iters"] == lm2["iters"]
    assert np.linalg.norm(x3 - x0) <= 1e-7 * np.linalg.norm(x0)
    # cap: stop the learned run early and finish with plain block-Jacobi
    x2, capped = api.solve(s, b, params=api.solve_params(precond=api.PRECOND_LEARNED, learned_cap=5, **prm))
    assert capped["fell_back"] and capped["converged"]
