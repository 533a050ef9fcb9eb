"""goal_avg_disp_noalloc (the avg disp functional from caller-owned device
arrays, partial sums in a fixed device array, no allocation) against the
regular functional path, goal_assemble with GOAL_NONE and GOAL_QOI_AVG_DISP.

Two calls in a row on different solutions (the second must not see the
first's partial sums), each within 1e-12 relative of the regular path (same
element arithmetic, another summation order), with the device's free memory
unchanged across them, and the host-side rejections
(too many elements, null pointers) that return before any launch. The file is
collected last so that it also runs after every other GPU test."""
import ctypes

import numpy as np
import pytest

from goal_gb300 import api, lib
from goal_gb300.mesh import kuhn_cube

pytestmark = pytest.mark.gpu

MAX_ELEMS = 16_777_216
GOAL_ERR_ARG, GOAL_ERR_CAPACITY = 1, 6  # include/goal_gb300.h


def _regular(mesh, U):
    d = api.Disc(mesh)
    m = api.Mechanics(d, api.NEOHOOKEAN, [[1000.0, 0.25, 0.0, 0.0, 0.0]])
    m.set_solution(U.ravel())
    return api.assemble(m, None, api.NONE, jacobian=False, save_states=False, qoi=api.QOI_AVG_DISP)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_matches_regular_functional_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    mesh = kuhn_cube(12)
    rng = np.random.default_rng(7)
    Us = [rng.standard_normal((mesh.num_nodes, 4)) * s for s in (1e-3, 5.0)]
    wants = [_regular(mesh, U) for U in Us]  # the regular path allocates: done before the checked calls
    X = torch.tensor(mesh.coords, dtype=torch.float64, device="cuda")
    T = torch.tensor(mesh.tets.astype(np.int32), dtype=torch.int32, device="cuda")
    J = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    Uds = [torch.tensor(U, dtype=torch.float64, device="cuda") for U in Us]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # a first call sets the entry point up on this device (the scratch
    # array's address, the kernels' module); the device's free memory must
    # then stay the same across the two checked calls
    rc = lib().goal_avg_disp_noalloc(_p(X), _p(T), _p(Uds[1]), mesh.num_nodes, mesh.num_elems, _p(J), stream)
    assert rc == 0, lib().goal_last_error()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    got = []
    for call in range(2):
        J.fill_(float("nan"))
        rc = lib().goal_avg_disp_noalloc(_p(X), _p(T), _p(Uds[call]), mesh.num_nodes, mesh.num_elems, _p(J), stream)
        assert rc == 0, lib().goal_last_error()
        torch.cuda.synchronize()
        got.append(J.item())
    assert torch.cuda.mem_get_info()[0] == free_before
    for call in range(2):
        want = wants[call]
        assert abs(got[call] - want) <= 1e-12 * max(abs(want), 1e-300), (call, got[call], want)


def test_rejects_without_launching():
    torch = pytest.importorskip("torch")
    mesh = kuhn_cube(2)
    X = torch.tensor(mesh.coords, dtype=torch.float64, device="cuda")
    T = torch.tensor(mesh.tets.astype(np.int32), dtype=torch.int32, device="cuda")
    U = torch.zeros((mesh.num_nodes, 4), dtype=torch.float64, device="cuda")
    J = torch.zeros(1, dtype=torch.float64, device="cuda")
    before = lib().goal_launch_count()
    rc = lib().goal_avg_disp_noalloc(_p(X), _p(T), _p(U), mesh.num_nodes, MAX_ELEMS + 1, _p(J), None)
    assert rc == GOAL_ERR_CAPACITY
    assert b"16777216" in lib().goal_last_error()
    rc = lib().goal_avg_disp_noalloc(None, _p(T), _p(U), mesh.num_nodes, mesh.num_elems, _p(J), None)
    assert rc == GOAL_ERR_ARG
    assert lib().goal_launch_count() == before
