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
