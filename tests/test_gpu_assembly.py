"""Parity of the CUDA element path with the oracle (calls through the C ABI).

Bars: DOF numbering and CSR graph bit-exact; residual, Jacobian and states
within 1e-12 relative (vectors: to the vector's max magnitude; matrices: to
each row's max magnitude); QoI values within 1e-12 relative; KS dMdu within
1e-10 relative: the reference differentiates von Mises through the stress after
the mixed pressure replacement (differences of diagonal entries that carry the
pressure) and, at plastic points, through the return-map iterates (which cancel
by a factor ~3 mubar/K); the closed-form derivative has neither cancellation,
so the two differ by the oracle's own rounding, measured at 7e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O
from goal_gb300 import api
from goal_gb300.mesh import kuhn_cube, graded_block

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel_vec(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def rel_rows(a, b, row_ptr):
    worst = 0.0
    for r in range(len(row_ptr) - 1):
        sl = slice(row_ptr[r], row_ptr[r + 1])
        scale = np.abs(b[sl]).max()
        if scale == 0:
            assert np.abs(a[sl]).max() == 0
            continue
        worst = max(worst, np.abs(a[sl] - b[sl]).max() / scale)
    return worst


def random_state(mesh, seed, u_scale, model):
    rng = np.random.default_rng(seed)
    u = u_scale * rng.standard_normal((mesh.num_nodes, 3))
    p = 50.0 * rng.standard_normal(mesh.num_nodes)
    st = O.States.initial(mesh.num_elems)
    if model == O.J2:
        for e in range(mesh.num_elems):
            G = 1e-3 * rng.standard_normal((3, 3))
            st.Fp_old[e] = O.expm(0.5 * (G + G.T)).ravel()
        st.eqps_old[:] = rng.uniform(0.0, 0.01, mesh.num_elems)
        st.Fp[:] = st.Fp_old
        st.eqps[:] = st.eqps_old
    st.sigma[:] = 100.0 * rng.standard_normal((mesh.num_elems, 9))
    st.sigma[:, [1, 2, 5]] = st.sigma[:, [3, 6, 7]]  # symmetric
    return u, p, st


MATS = {O.NEOHOOKEAN: O.Material(1000.0, 0.25, c0=1.0), O.J2: O.Material(200e3, 0.3, K=1000.0, Y=250.0, c0=1.0)}


def make_gpu(mesh, model, u, p, st):
    d = api.Disc(mesh)
    m = api.Mechanics(d, model, [MATS[model].row()])
    U = np.zeros((mesh.num_nodes, 4))
    U[:, :3] = u
    U[:, 3] = p
    m.set_solution(U.ravel())
    m.set_state(api.FP_OLD, st.Fp_old)
    m.set_state(api.EQPS_OLD, st.eqps_old)
    m.set_state(api.FP, st.Fp)
    m.set_state(api.EQPS, st.eqps)
    m.set_state(api.SIGMA, st.sigma)
    s = api.SolInfo(d)
    return d, m, s


@pytest.fixture(scope="module")
def meshes(cube_kat):
    return {"cube_kat": cube_kat[0], "kuhn3": kuhn_cube(3), "graded": graded_block(3000, seed=2)}


@pytest.mark.parametrize("name", ["cube_kat", "kuhn3", "graded"])
def test_graph_bit_exact(meshes, name):
    mesh = meshes[name]
    d = api.Disc(mesh)
    rp, ci = d.graph()
    orp, oci = O.csr_graph(mesh.num_nodes, mesh.tets)
    assert np.array_equal(rp, orp)
    assert np.array_equal(ci, oci)
    assert d.nnz == len(oci)


@pytest.mark.parametrize("name", ["cube_kat", "kuhn3", "graded"])
def test_coloring_is_valid(meshes, name):
    mesh = meshes[name]
    d = api.Disc(mesh)
    col = d.colors()
    assert col.min() == 0 and col.max() == d.num_colors - 1
    for c in range(d.num_colors):
        nodes = mesh.tets[col == c].ravel()
        assert len(np.unique(nodes)) == len(nodes), f"colour {c} shares nodes"
    # the build's phase times: every phase ran, the colouring took at least
    # one Jones-Plassmann round per colour beyond the first
    bt = d.build_times()
    assert all(bt[k] >= 0.0 for k in ("graph", "colouring", "layout", "contribution_lists", "sets"))
    assert bt["colour_rounds"] >= d.num_colors


@pytest.mark.parametrize("colored", [False, True])
@pytest.mark.parametrize("model,u_scale", [(O.NEOHOOKEAN, 0.02), (O.J2, 2e-4), (O.J2, 2e-3)])
def test_primal_jacobian_chain(meshes, model, u_scale, colored):
    mesh = meshes["kuhn3"]
    u, p, st = random_state(mesh, 11, u_scale, model)
    d, m, s = make_gpu(mesh, model, u, p, st)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=True, colored=colored)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    ost = st.copy()
    _, npl = O.assemble(mesh, model, [MATS[model]], u, p, ost, mode=O.PRIMAL, fad=True, save=True, graph=g, R=R,
                        vals=vals)
    assert rel_vec(s.R, R) < RTOL
    assert rel_rows(s.dRdu_csr(), vals, g[0]) < RTOL
    assert rel_vec(m.get_state(api.SIGMA), ost.sigma) < RTOL
    if model == O.J2:
        assert rel_vec(m.get_state(api.EQPS), ost.eqps) < RTOL
        assert rel_vec(m.get_state(api.FP), ost.Fp) < RTOL
        if u_scale > 1e-3:
            assert npl > 0


@pytest.mark.parametrize("model", [O.NEOHOOKEAN, O.J2])
def test_residual_chain(meshes, model):
    mesh = meshes["cube_kat"]
    u, p, st = random_state(mesh, 5, 0.01 if model == O.NEOHOOKEAN else 1e-3, model)
    d, m, s = make_gpu(mesh, model, u, p, st)
    api.assemble(m, s, api.PRIMAL, jacobian=False, save_states=True)
    R = np.zeros(4 * mesh.num_nodes)
    ost = st.copy()
    O.assemble(mesh, model, [MATS[model]], u, p, ost, mode=O.PRIMAL, fad=False, save=True, R=R)
    assert rel_vec(s.R, R) < RTOL
    assert rel_vec(m.get_state(api.SIGMA), ost.sigma) < RTOL


@pytest.mark.parametrize("colored", [False, True])
@pytest.mark.parametrize("model,qoi", [(O.NEOHOOKEAN, O.QOI_AVG_DISP), (O.NEOHOOKEAN, O.QOI_KS),
                                       (O.J2, O.QOI_AVG_DISP), (O.J2, O.QOI_KS)])
def test_adjoint_chain(meshes, model, qoi, colored):
    mesh = meshes["kuhn3"]
    u, p, st = random_state(mesh, 7, 0.02 if model == O.NEOHOOKEAN else 1e-3, model)
    # stored stresses that the KS pre-pass reads: the model's own stresses
    ost0 = st.copy()
    O.assemble(mesh, model, [MATS[model]], u, p, ost0, mode=O.PRIMAL, fad=False, save=True, R=np.zeros(4 * mesh.num_nodes))
    st.sigma[:] = ost0.sigma * 1.05
    d, m, s = make_gpu(mesh, model, u, p, st)
    rho = 20.0
    q = api.assemble(m, s, api.ADJOINT, jacobian=True, save_states=False, qoi=qoi, rho=rho, colored=colored)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    dM = np.zeros(4 * mesh.num_nodes)
    oq, _ = O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.ADJOINT, fad=True, save=False, graph=g,
                       R=R, vals=vals, dMdu=dM, qoi=qoi, rho=rho)
    assert rel_vec(s.R, R) < RTOL
    assert rel_rows(s.dRdu_csr(), vals, g[0]) < RTOL
    assert abs(q - oq) <= RTOL * abs(oq)
    tol = 1e-10 if qoi == O.QOI_KS else RTOL
    assert rel_vec(s.dMdu, dM) < tol


@pytest.mark.parametrize("model,qoi", [(O.NEOHOOKEAN, O.QOI_AVG_DISP), (O.J2, O.QOI_KS)])
def test_functional_chain(meshes, model, qoi):
    mesh = meshes["graded"]
    u, p, st = random_state(mesh, 9, 0.01 if model == O.NEOHOOKEAN else 1e-3, model)
    d, m, s = make_gpu(mesh, model, u, p, st)
    q = api.assemble(m, None, api.NONE, jacobian=False, save_states=False, qoi=qoi, rho=20.0)
    oq, _ = O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.NONE, fad=False, save=False, qoi=qoi,
                       rho=20.0)
    assert abs(q - oq) <= RTOL * abs(oq)


@pytest.mark.parametrize("model", [O.NEOHOOKEAN, O.J2])
def test_error_chain(meshes, model):
    mesh = meshes["kuhn3"]
    u, p, st = random_state(mesh, 13, 0.01 if model == O.NEOHOOKEAN else 1e-3, model)
    rng = np.random.default_rng(3)
    zd = rng.standard_normal((mesh.num_nodes, 4))
    zc = rng.standard_normal((mesh.num_nodes, 4))
    d, m, s = make_gpu(mesh, model, u, p, st)
    m.set_weights(zd.ravel(), zc.ravel())
    api.assemble(m, s, api.PRIMAL, jacobian=False, save_states=False, error_chain=True)
    R = np.zeros(4 * mesh.num_nodes)
    O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.PRIMAL, fad=False, save=False, R=R,
               error_weights=(np.ascontiguousarray(zd[:, :3]), np.ascontiguousarray(zd[:, 3]),
                              np.ascontiguousarray(zc[:, 3])))
    assert rel_vec(s.R, R) < RTOL
    # traction with the DWR weights
    bcs = api.Bcs(d, traction=[("xmax", "10.0", "1.0*t", "x*y")])
    R0 = s.R
    api.set_tbcs(m, s, bcs, 2.0, error_weights=True)
    O.apply_tbcs(mesh, [O.TBC("xmax", ("10.0", "1.0*t", "x*y"))], 2.0, R, zu=np.ascontiguousarray(zd[:, :3]))
    assert rel_vec(s.R - R0, R - R0) < RTOL


def test_boundary_conditions(meshes):
    mesh = meshes["kuhn3"]
    model = O.J2
    u, p, st = random_state(mesh, 17, 1e-3, model)
    d, m, s = make_gpu(mesh, model, u, p, st)
    dbcs = [(0, "xmin", "0.0"), (1, "ymin", "0.0"), (2, "zmin", "0.0"), (0, "xmax", "0.002*t")]
    tbcs = [("ymax", "0.0", "1.0*t", "0.5*sin(x)")]
    bcs = api.Bcs(d, dbcs, tbcs)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False)
    api.set_tbcs(m, s, bcs, 3.0)
    api.set_jac_dbcs(m, s, bcs, 3.0)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    dM = np.zeros(4 * mesh.num_nodes)
    O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.PRIMAL, fad=True, save=False, graph=g, R=R,
               vals=vals, dMdu=dM)
    O.apply_tbcs(mesh, [O.TBC(*([t[0]] + [tuple(t[1:])])) for t in tbcs], 3.0, R)
    O.apply_dbcs(mesh, [O.DBC(*b) for b in dbcs], 3.0, u, R, g, vals, dM, jac=True)
    assert rel_vec(s.R, R) < RTOL
    assert rel_rows(s.dRdu_csr(), vals, g[0]) < RTOL
    assert np.all(s.dMdu == dM)
    # residual-only DBCs
    api.assemble(m, s, api.PRIMAL, jacobian=False, save_states=False)
    api.set_resid_dbcs(m, s, bcs, 3.0)
    R2 = np.zeros(4 * mesh.num_nodes)
    O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.PRIMAL, fad=False, save=False, R=R2)
    O.apply_dbcs(mesh, [O.DBC(*b) for b in dbcs], 3.0, u, R2)
    assert rel_vec(s.R, R2) < RTOL


@pytest.mark.parametrize("name", ["cube_kat", "kuhn3", "graded"])
def test_nested_mesh_matches_oracle(meshes, name):
    mesh = meshes[name]
    d = api.Disc(mesh)
    n = d.nested()
    X, T, ES = n.get_mesh()
    on, edges, parent = O.refine_uniform(mesh)
    assert np.array_equal(n.parent_edges(), edges)
    assert np.array_equal(X, on.coords)
    assert np.array_equal(T, on.tets)
    assert np.array_equal(ES, on.elem_set)
    rp, ci = n.graph()
    orp, oci = O.csr_graph(on.num_nodes, on.tets)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)


@pytest.mark.parametrize("colored", [False, True])
def test_assembly_is_deterministic_and_overwrite_matches_accumulate(meshes, colored):
    mesh = meshes["graded"]
    u, p, st = random_state(mesh, 19, 1e-3, O.J2)
    d, m, s = make_gpu(mesh, O.J2, u, p, st)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, colored=colored)
    R1, A1 = s.R, s.dRdu_bsr()
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, colored=colored)
    assert np.array_equal(R1, s.R) and np.array_equal(A1, s.dRdu_bsr())
    s.zero_all()
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, overwrite=False, colored=colored)
    assert np.array_equal(R1, s.R)
    if colored:
        assert np.array_equal(A1, s.dRdu_bsr())
    else:
        # accumulating sums every block from its element blocks; overwriting
        # forms the diagonal blocks' u columns from the rows' off-diagonal blocks
        assert np.abs(s.dRdu_bsr() - A1).max() <= 1e-13 * np.abs(A1).max()
    # both scatter strategies assemble the same matrix (up to summation order)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False, colored=not colored)
    assert np.abs(s.dRdu_bsr() - A1).max() <= 1e-13 * np.abs(A1).max()


def _gpu_with_mats(mesh, model, mats, u, p, st, stabilization=True):
    d = api.Disc(mesh)
    m = api.Mechanics(d, model, [mt.row() for mt in mats], stabilization=stabilization)
    U = np.zeros((mesh.num_nodes, 4))
    U[:, :3] = u
    U[:, 3] = p
    m.set_solution(U.ravel())
    m.set_state(api.FP_OLD, st.Fp_old)
    m.set_state(api.EQPS_OLD, st.eqps_old)
    m.set_state(api.FP, st.Fp)
    m.set_state(api.EQPS, st.eqps)
    m.set_state(api.SIGMA, st.sigma)
    return d, m, api.SolInfo(d)


@pytest.mark.parametrize("model", [O.NEOHOOKEAN, O.J2])
@pytest.mark.parametrize("stabilization", [True, False])
def test_heterogeneous_materials(model, stabilization):
    """Per-element-set materials (four regions of a graded block, different E,
    nu, Y, c0), with and without the stabilization term."""
    mesh = graded_block(2500, seed=5, regions=4)
    assert len(np.unique(mesh.elem_set)) == 4
    rng = np.random.default_rng(3)
    mats = [O.Material(float(rng.lognormal(np.log(1000.0), 0.5)), float(rng.uniform(0.2, 0.45)), K=100.0,
                       Y=float(rng.uniform(5.0, 30.0)), c0=float(rng.uniform(0.5, 2.0))) for _ in range(4)]
    u, p, st = random_state(mesh, 17, 0.02 if model == O.NEOHOOKEAN else 5e-3, model)
    d, m, s = _gpu_with_mats(mesh, model, mats, u, p, st, stabilization)
    api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=True)
    g = O.csr_graph(mesh.num_nodes, mesh.tets)
    R = np.zeros(4 * mesh.num_nodes)
    vals = np.zeros(len(g[1]))
    ost = st.copy()
    _, npl = O.assemble(mesh, model, mats, u, p, ost, mode=O.PRIMAL, fad=True, save=True, graph=g, R=R, vals=vals,
                        stabilization=stabilization)
    assert rel_vec(s.R, R) < RTOL
    assert rel_rows(s.dRdu_csr(), vals, g[0]) < RTOL
    if model == O.J2:
        assert npl > 0
        assert rel_vec(m.get_state(api.FP), ost.Fp) < RTOL


def test_single_element_and_single_colour():
    """The smallest mesh: one tet (one colour, one 16x16 element matrix)."""
    from goal_gb300.mesh import Mesh
    coords = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    tets = np.array([[0, 1, 2, 3]], np.int32)
    mesh = Mesh(coords=coords, tets=tets, elem_set=np.zeros(1, np.int32), elem_set_names=["one"],
                node_sets={"xmin": np.array([0, 2, 3], np.int32)}, side_sets={})
    for model in (O.NEOHOOKEAN, O.J2):
        u, p, st = random_state(mesh, 2, 0.05, model)
        d, m, s = make_gpu(mesh, model, u, p, st)
        assert d.num_colors == 1
        api.assemble(m, s, api.PRIMAL, jacobian=True, save_states=False)
        g = O.csr_graph(mesh.num_nodes, mesh.tets)
        R = np.zeros(16)
        vals = np.zeros(len(g[1]))
        O.assemble(mesh, model, [MATS[model]], u, p, st.copy(), mode=O.PRIMAL, fad=True, save=False, graph=g, R=R,
                   vals=vals)
        assert len(vals) == 256
        assert rel_vec(s.R, R) < RTOL
        assert rel_rows(s.dRdu_csr(), vals, g[0]) < RTOL


def test_measured_fp64_peak_is_plausible():
    """The FP64 roofline's denominator: GB300 issues 2 FP64 FMAs per clock per
    SM (1.26 TFLOP/s at 2.07 GHz on 152 SMs)."""
    import ctypes
    from goal_gb300 import lib
    v = ctypes.c_double()
    assert lib().goal_measure_fp64_peak(ctypes.byref(v)) == 0
    assert 0.5 < v.value < 2.0, v.value


@pytest.mark.parametrize("mode", [api.PRIMAL, api.ADJOINT])
def test_chunked_element_buffer_same_bits(mode):
    """With the element buffer capped (goal_set_element_buffer_limit) the
    two-phase assembly runs in chunks of elements; R, the matrix blocks and
    dM/du are the same bits as one pass over all elements, and the one-pass
    default (diagonal blocks formed from the rows' off-diagonal blocks) agrees
    with both to 1e-13 of each row's largest entry."""
    from goal_gb300 import lib
    mesh = kuhn_cube(5)
    u, p, st = random_state(mesh, 11, 1e-3, O.J2)
    d, m, s = make_gpu(mesh, api.J2, u, p, st)
    qoi = api.QOI_AVG_DISP if mode == api.ADJOINT else api.QOI_NONE
    # one pass, every block summed from its element blocks (accumulating into zeros)
    s.zero_all()
    api.assemble(m, s, mode, jacobian=True, save_states=False, qoi=qoi, overwrite=False)
    R1, A1, M1, C1 = s.R, s.dRdu_bsr(), s.dMdu, s.dRdu_csr()
    # default: one pass, diagonal blocks from row sums
    api.assemble(m, s, mode, jacobian=True, save_states=False, qoi=qoi)
    C0 = s.dRdu_csr()
    try:
        assert lib().goal_set_element_buffer_limit(7 * 2304 * 8) == 0  # chunks of about 60 of the 750 elements
        s2 = api.SolInfo(d)
        api.assemble(m, s2, mode, jacobian=True, save_states=False, qoi=qoi)
        assert np.array_equal(s2.R, R1) and np.array_equal(s2.dRdu_bsr(), A1) and np.array_equal(s2.dMdu, M1)
    finally:
        lib().goal_set_element_buffer_limit(0)
    assert rel_rows(C0, C1, d.graph()[0]) <= 1e-13
