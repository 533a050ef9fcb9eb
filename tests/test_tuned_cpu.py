"""The tuned CPU baseline (oracle/tuned.cpp: closed-form tangent, coloured
OpenMP) assembles the same primal Jacobian chain as the dual-number oracle:
R, every Jacobian row and the state writes within 1e-12 relative, for J2 (half
of the points plastic) and neo-Hookean, with stabilization."""
import numpy as np
import pytest

from oracle import oracle as O
from goal_gb300.mesh import kuhn_cube


def _state(mesh, seed, plastic):
    rng = np.random.default_rng(seed)
    u = 1e-3 * rng.standard_normal((mesh.num_nodes, 3)) * (3.0 if plastic else 1.0)
    p = 50.0 * rng.standard_normal(mesh.num_nodes)
    st = O.States.initial(mesh.num_elems)
    for e in range(mesh.num_elems):
        G = 1e-3 * rng.standard_normal((3, 3))
        st.Fp_old[e] = O.expm(0.5 * (G + G.T)).ravel()
    st.eqps_old[:] = rng.uniform(0.0, 0.01, mesh.num_elems)
    st.Fp[:] = st.Fp_old
    st.eqps[:] = st.eqps_old
    return u, p, st


def _rows(a, b, row_ptr):
    worst = 0.0
    for r in range(len(row_ptr) - 1):
        sl = slice(row_ptr[r], row_ptr[r + 1])
        scale = np.abs(b[sl]).max()
        worst = max(worst, np.abs(a[sl] - b[sl]).max() / scale if scale > 0 else np.abs(a[sl]).max())
    return worst


@pytest.mark.parametrize("model", [O.J2, O.NEOHOOKEAN])
def test_tuned_matches_oracle(model):
    mesh = kuhn_cube(4, jitter=0.2, seed=3)
    mat = O.Material(200e3, 0.3, K=1000.0, Y=250.0, c0=1.0) if model == O.J2 else O.Material(1000.0, 0.25, c0=1.0)
    u, p, st = _state(mesh, 5, model == O.J2)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    ost = st.copy()
    _, npl = O.assemble(mesh, model, [mat], u, p, ost, mode=O.PRIMAL, fad=True, save=True, graph=g, R=R, vals=vals)
    T = O.TunedAssembly(mesh, model, [mat], st.Fp_old)
    T.Fp[:] = st.Fp
    U = np.zeros((mesh.num_nodes, 4))
    U[:, :3] = u
    U[:, 3] = p
    assert T.assemble(U, st.eqps_old) == 0
    assert np.abs(T.R - R).max() <= 1e-12 * np.abs(R).max()
    assert _rows(T.csr_values(), vals, g[0]) <= 1e-12
    assert np.abs(T.sigma - ost.sigma).max() <= 1e-12 * np.abs(ost.sigma).max()
    if model == O.J2:
        assert npl > mesh.num_elems // 4
        assert np.abs(T.eqps - ost.eqps).max() <= 1e-14
        assert np.abs(T.Fp - ost.Fp).max() <= 1e-12
