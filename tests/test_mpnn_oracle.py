"""The numpy restatement of the learned block-Jacobi correction (oracle/mpnn.py)
on its own: the loss gradient against central finite differences (weights
unrounded, float64 parameters), the untrained network being plain
block-Jacobi, and the Dirichlet rows staying untouched. The CUDA kernels are
compared with this restatement in the GPU tests."""
import numpy as np
import pytest

from oracle import mpnn as M
from oracle import oracle as O


def _system(cube_kat):
    mesh, _ = cube_kat
    rng = np.random.default_rng(2)
    u = 0.01 * rng.standard_normal((mesh.num_nodes, 3))
    p = rng.standard_normal(mesh.num_nodes)
    st = O.States.initial(mesh.num_elems)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    n = 4 * mesh.num_nodes
    R = np.zeros(n)
    vals = np.zeros(len(g[1]))
    mat = O.Material(1000.0, 0.25, K=100.0, Y=10.0, c0=1.0)
    O.assemble(mesh, O.J2, [mat], u, p, st, mode=O.PRIMAL, fad=True, save=False, graph=g, R=R, vals=vals)
    O.apply_dbcs(mesh, [O.DBC(0, "xmin", "0.0"), O.DBC(1, "xmin", "0.0")], 0.0, u, R, g, vals, None, jac=True)
    A = O.csr_matrix(g, vals, n).tobsr(blocksize=(4, 4))
    A.sort_indices()
    brow, bcol, blk = A.indptr, A.indices, A.data
    diag = np.array([brow[k] + np.searchsorted(bcol[brow[k]:brow[k + 1]], k) for k in range(mesh.num_nodes)])
    return brow, bcol, diag, blk


def test_untrained_network_is_block_jacobi(cube_kat):
    brow, bcol, diag, A = _system(cube_kat)
    x, e, sd, Dinv, dirichlet = M.features(brow, bcol, diag, A)
    assert dirichlet.any()
    C = M.forward(M.unflatten(M.init_params(0)), brow, bcol, diag, x, e)
    assert np.all(C == 0)
    r = np.random.default_rng(0).standard_normal(4 * len(diag))
    B = M.blocks(C, sd, Dinv, dirichlet)
    assert np.array_equal(M.apply_P(brow, bcol, A, Dinv, B, r),
                          np.einsum("nij,nj->ni", Dinv, r.reshape(-1, 4)).ravel())


def test_dirichlet_rows_untouched(cube_kat):
    brow, bcol, diag, A = _system(cube_kat)
    x, e, sd, Dinv, dirichlet = M.features(brow, bcol, diag, A)
    C = np.random.default_rng(1).standard_normal((len(diag), 16)).astype(np.float32)
    B = M.blocks(C, sd, Dinv, dirichlet)
    assert np.all(B[dirichlet] == 0)   # rows of Dirichlet dofs
    r = np.random.default_rng(3).standard_normal(4 * len(diag))
    z = np.einsum("nij,nj->ni", Dinv, r.reshape(-1, 4))
    Pr = M.apply_P(brow, bcol, A, Dinv, B, r).reshape(-1, 4)
    assert np.array_equal(Pr[dirichlet], z[dirichlet])


def test_gradient_matches_finite_differences(cube_kat, monkeypatch):
    monkeypatch.setattr(M, "ROUND_BF16", False)
    brow, bcol, diag, A = _system(cube_kat)
    rng = np.random.default_rng(5)
    theta = M.init_params(1).astype(np.float64) + 0.05 * rng.standard_normal(M.num_params())
    probes = [rng.standard_normal(4 * len(diag)) for _ in range(2)]

    def loss(t):
        # float64 parameters through the float32 network: use a float64 copy of the module's path
        return M.loss_and_grad(t, brow, bcol, diag, A, probes)[0]

    L0, g = M.loss_and_grad(theta, brow, bcol, diag, A, probes)
    assert L0 > 0
    for k in range(4):
        d = rng.standard_normal(M.num_params())
        d /= np.linalg.norm(d)
        h = 1e-2
        fd = (loss(theta + h * d) - loss(theta - h * d)) / (2 * h)
        an = g @ d
        assert abs(fd - an) <= 2e-2 * max(abs(an), 1e-3 * np.linalg.norm(g)), (k, fd, an)
