"""Parity at the production size: the benchmark's own workload (J2 mixed u-p
on the Kuhn cube 40^3, 384,000 tets, 15.9M matrix entries, half of the points
plastic) assembled on the GPU and by the oracle (all host cores), compared
entry by entry: R 1e-12 of its max, every Jacobian row 1e-12 of its row max,
the states 1e-12. Also the determinism of the GPU path at that size (two
assemblies, bitwise equal)."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from goal_gb300 import api

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RTOL = 1e-12


def test_bench_workload_matches_oracle_entrywise():
    sys.path.insert(0, ROOT)
    import bench
    mesh, u, p, Fp_old, eqps_old, amp, frac = bench.workload(40)
    assert mesh.num_elems == 384000 and abs(frac - 0.5) < 0.01
    M = bench.MAT
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.J2, [[M["E"], M["nu"], M["K"], M["Y"], M["c0"]]])
    U = np.zeros((mesh.num_nodes, 4))
    U[:, :3] = u
    U[:, 3] = p
    m.set_solution(U.ravel())
    m.set_state(api.FP_OLD, Fp_old)
    m.set_state(api.EQPS_OLD, eqps_old)
    s = api.SolInfo(d)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=True)
    R1, V1 = s.R.copy(), s.dRdu_bsr().copy()
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=True)
    assert np.array_equal(s.R, R1) and np.array_equal(s.dRdu_bsr(), V1)

    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    st = O.States.initial(mesh.num_elems)
    st.Fp_old[:] = Fp_old
    st.eqps_old[:] = eqps_old
    mat = O.Material(M["E"], M["nu"], K=M["K"], Y=M["Y"], c0=M["c0"])
    _, npl = O.assemble(mesh, O.J2, [mat], u, p, st, mode=O.PRIMAL, fad=True, save=True, graph=g, R=R, vals=vals,
                        threads=True)
    assert npl > 0.4 * mesh.num_elems
    assert np.abs(s.R - R).max() <= RTOL * np.abs(R).max()
    # row-relative Jacobian comparison, vectorized over the CSR rows
    rp = g[0]
    gv = s.dRdu_csr()
    rowmax = np.maximum.reduceat(np.abs(vals), rp[:-1])
    rowerr = np.maximum.reduceat(np.abs(gv - vals), rp[:-1])
    assert np.all(rowerr <= RTOL * np.maximum(rowmax, 1e-300))
    for which, ref in ((api.EQPS, st.eqps), (api.FP, st.Fp), (api.SIGMA, st.sigma)):
        got = m.get_state(which)
        assert np.abs(got - ref).max() <= RTOL * np.abs(ref).max()
