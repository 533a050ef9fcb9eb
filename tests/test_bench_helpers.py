"""Host-side helpers of bench.py that need no GPU: the element count a size
field asks for, and the adaptive leg keeping its finished cycles when a later
cycle fails."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from goal_gb300.mesh import kuhn_cube  # noqa: E402


def _mean_rms_edge(mesh):
    x, t = mesh.coords, mesh.tets
    h2 = sum(((x[t[:, a]] - x[t[:, b]]) ** 2).sum(axis=1) for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)))
    return np.sqrt(h2 / 6.0)


def test_field_elements_counts_the_requested_refinement():
    mesh = kuhn_cube(6)
    h = _mean_rms_edge(mesh)
    # on the Kuhn grid every tet has the same rms edge length
    assert np.allclose(h, h[0])
    same = np.full(mesh.num_nodes, h[0])
    assert bench._field_elements(mesh, same) == pytest.approx(mesh.num_elems)
    # half the size asks for 8x the elements, twice the size for 1/8
    assert bench._field_elements(mesh, same / 2) == pytest.approx(8 * mesh.num_elems)
    assert bench._field_elements(mesh, same * 2) == pytest.approx(mesh.num_elems / 8)
    # a field graded in x: the count is the sum of the per-element ratios cubed
    size = h[0] * (1.0 + mesh.coords[:, 0])
    ht = size[mesh.tets].mean(axis=1)
    assert bench._field_elements(mesh, size) == pytest.approx(((h / ht) ** 3).sum())


def test_adaptive_leg_keeps_finished_cycles(monkeypatch):
    def fake_leg(api, cycles, start, records=None, **kw):
        records.append({"cycle": 0, "elements": start})
        records.append({"cycle": 1, "elements": 2 * start})
        raise RuntimeError("out of memory in cycle 2")

    monkeypatch.setattr(bench, "adaptive_leg", fake_leg)
    out = bench.adaptive_leg_partial(None, 6, 1000)
    assert [r.get("cycle") for r in out[:2]] == [0, 1]
    assert out[2] == {"error": "out of memory in cycle 2"}


def test_adaptive_leg_partial_passes_results_through(monkeypatch):
    monkeypatch.setattr(bench, "adaptive_leg", lambda api, *a, records=None, **kw: [{"cycle": 0}])
    assert bench.adaptive_leg_partial(None, 1, 10) == [{"cycle": 0}]


class _FakeApi:
    """Stands in for goal_gb300.api in bench._j2_ramp: a Newton solve fails
    when its load increment exceeds ``max_inc``; calls are recorded."""

    J2 = MIXED = NONE = QOI_KS_VM = 0

    class GoalError(RuntimeError):
        pass

    def __init__(self, max_inc):
        self.max_inc = max_inc
        self.calls = []
        api = self

        class Mechanics:
            def __init__(self, d, model, mats, fp_reset=False):
                self.U = np.zeros(4)
                self.updates = 0

            def set_line_search(self, k):
                pass

            def update_states(self):
                self.updates += 1
                api.calls.append(("update",))

            def get_solution(self):
                return self.U.copy()

            def set_solution(self, U):
                self.U = np.asarray(U, dtype=float).copy()
                api.calls.append(("restore", float(self.U[0])))

        self.Mechanics = Mechanics
        self.Disc = lambda mesh: object()
        self.SolInfo = lambda d: object()
        self.Bcs = lambda d, dbcs, tbcs: object()

    @staticmethod
    def solve_params(**kw):
        return kw

    def primal_solve(self, m, s, bcs, t_now, t_old, max_iters, tol, prm):
        self.calls.append(("solve", t_old, t_now))
        if t_now - t_old > self.max_inc + 1e-12:
            m.U[:] = -1.0  # a diverged iterate
            e = self.GoalError("newton failed")
            e.stats = {"norms": [1.0] * max_iters}
            raise e
        m.U[:] = t_now
        return {"iters": 3, "linear_iters": 30, "backtracks": 0}

    def assemble(self, *a, **kw):
        return 0.0


def test_ramp_cutbacks_halve_failed_increments_and_grow_back():
    api = _FakeApi(max_inc=0.5)
    *_, out = bench._j2_ramp(api, 2, 3, max_newton=12, cutbacks=6, jitter=0.0)
    # step 1: 1.0 fails, then 0.5 + 0.5; step 2: 0.5 x 2; the fourth success
    # in a row (the end of step 2) lets step 3 try a full step, which fails,
    # and step 3 ends in halves
    solves = [c[1:] for c in api.calls if c[0] == "solve"]
    assert solves[0] == (0.0, 1.0)
    assert (0.0, 0.5) in solves and (0.5, 1.0) in solves
    assert out["substeps"] == [2, 2, 2]
    # Newton iterations per load step: the failed attempt's 12 plus 3 per substep
    assert out["iters"][0] == 12 + 2 * 3
    # a failed attempt restores the solution it started from
    restores = [c[1] for c in api.calls if c[0] == "restore"]
    assert restores and all(r >= 0.0 for r in restores)
    # the states are updated once before every solve that follows a success
    seq = [c[0] for c in api.calls]
    for i, c in enumerate(seq):
        if c == "update":
            assert seq[i + 1] == "solve"


def test_ramp_without_cutbacks_is_goals_newton():
    api = _FakeApi(max_inc=0.5)
    with pytest.raises(_FakeApi.GoalError) as exc:
        bench._j2_ramp(api, 2, 3, cutbacks=0, jitter=0.0)
    assert exc.value.step == 1
    assert [c[0] for c in api.calls] == ["solve"]


def test_ramp_gives_up_after_its_cutbacks():
    api = _FakeApi(max_inc=0.1)
    with pytest.raises(_FakeApi.GoalError) as exc:
        bench._j2_ramp(api, 2, 2, cutbacks=2, jitter=0.0)
    assert exc.value.step == 1
    incs = [c[2] - c[1] for c in api.calls if c[0] == "solve"]
    assert incs == [1.0, 0.5, 0.25]
