"""goal's full Newton (src/goal_primal.cpp:111-137: no line search, absolute
tolerance, failure aborts the run) on the J2 stretched cube of the
production-size configuration (E = 200e3, nu = 0.3, Y = 250, K = 1000, c0 = 1;
u = 0 on x = 0, u_x = inc t on x = 1), run on the oracle (direct linear
solves) on a jittered 8^3 Kuhn cube.

With the configuration's increment of 0.002 per load step (u_x = 0.02 in 10
steps) the third step diverges: the residual grows every iteration until the
return map sees non-finite strains. With 0.0005 per step every step converges
in 7 iterations or fewer on this mesh (a full run to u_x = 0.02, 40 steps,
converges throughout).

On this mesh the cause is goal's J2 state write (src/goal_J2.cpp:97-136): Fp
is written only at points that yield, so at a point that is plastic in an
early Newton iterate and elastic at convergence the early iterate's Fp
survives, and States::update commits it as Fp_old. With the Fp_old reset
option (Fp = Fp_old at elastic points; off by default, goal's behaviour
otherwise) the configuration's own ramp converges in 7 or 8 iterations per
step. Finer meshes need more: the same full Newton with the reset reproduces
the oracle's iterates on the 16^3 cube and converges there, but stops at the
second step on the 24^3 cube and at the first on the 40^3 cube, where only
halving the failed load increments (a driver-level cutback, not in goal)
carries the ramp to u_x = 0.02."""
import numpy as np
import pytest

from oracle import oracle as O
from goal_gb300.mesh import kuhn_cube

MAT = O.Material(200e3, 0.3, K=1000.0, Y=250.0, c0=1.0)


def _primal(inc, fp_reset=False):
    mesh = kuhn_cube(8, jitter=0.2, seed=1)
    dbcs = [O.DBC(0, "xmin", "0.0"), O.DBC(1, "xmin", "0.0"), O.DBC(2, "xmin", "0.0"), O.DBC(0, "xmax", f"{inc}*t")]
    return O.Primal(O.Problem(mesh, O.J2, [MAT], dbcs, [], qoi=O.QOI_KS, rho=20.0, fp_reset=fp_reset))


def _ramp(P, steps, max_iters=15):
    """Load steps t = 1..steps with States::update between them; returns the
    Newton iteration counts, and the failing step (or None)."""
    its = []
    for k in range(1, steps + 1):
        if k > 1:
            P.states.update()
        try:
            with np.errstate(all="ignore"):
                its.append(len(P.solve(float(k), float(k - 1), max_iters=max_iters, tol=1e-8)))
        except RuntimeError:
            return its, k
    return its, None


@pytest.mark.filterwarnings("ignore::scipy.sparse.linalg.MatrixRankWarning")
def test_configured_increment_diverges():
    its, failed = _ramp(_primal(0.002), 3)
    assert failed == 3, (its, failed)
    assert its[:2] == [8, 8]


def test_quarter_increment_converges():
    P = _primal(0.0005)
    its, failed = _ramp(P, 8)
    assert failed is None
    assert max(its) <= 7
    assert P.states.eqps.max() > 0.002  # plastic flow well past first yield (u_x = 0.004)


def test_configured_increment_converges_with_fp_reset():
    P = _primal(0.002, fp_reset=True)
    its, failed = _ramp(P, 4)
    assert failed is None
    assert max(its) <= 8
