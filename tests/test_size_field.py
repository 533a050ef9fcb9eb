"""Target size field (src/goal_size_field.cpp): the restatement's closed-form
properties on the CPU, and the CUDA kernels against the restatement (1e-13
relative: same formula, pow and summation order differ) on the GPU."""
import numpy as np
import pytest

from goal_gb300.mesh import kuhn_cube
from oracle import size_field as SF


def test_uniform_error_scales_the_mesh_size():
    mesh = kuhn_cube(4)
    h = SF.element_sizes(mesh.coords, mesh.tets)
    E = mesh.num_elems
    # equal indicators: h_new = (E / target)^(1/3) h, whatever the indicator value
    for target, theta in ((E, 3.7), (8 * E, 1e-6), (E // 8, 0.2)):
        hn_expected = np.clip((E / target) ** (1.0 / 3.0) * h, 0.25 * h, 2.0 * h)
        s = SF.iso_target_size(mesh.coords, mesh.tets, np.full(E, theta), target)
        # every Kuhn tet has the same edge lengths (3 x h, 2 x sqrt2 h, 1 x sqrt3 h)
        assert np.allclose(s, hn_expected.mean(), rtol=1e-12)


def test_clamps_to_quarter_and_double():
    mesh = kuhn_cube(3)
    E = mesh.num_elems
    err = np.ones(E)
    err[0] = 0.0        # zero error: size grows to the upper clamp
    err[1] = 1e12       # huge error: size shrinks to the lower clamp
    h = SF.element_sizes(mesh.coords, mesh.tets)
    s = SF.iso_target_size(mesh.coords, mesh.tets, err, E)
    assert np.all(np.isfinite(s))
    assert s.max() <= 2.0 * h.max() + 1e-15 and s.min() >= 0.25 * h.min() - 1e-15


@pytest.mark.gpu
def test_gpu_matches_restatement():
    from goal_gb300 import api
    for mesh in (kuhn_cube(6, jitter=0.2, seed=3), kuhn_cube(5)):
        d = api.Disc(mesh)
        rng = np.random.default_rng(0)
        err = rng.lognormal(-6.0, 2.0, mesh.num_elems) * rng.choice([-1.0, 1.0], mesh.num_elems)
        err[::97] = 0.0
        for target in (100, mesh.num_elems, 10 * mesh.num_elems):
            got = api.size_field(d, err, target)
            want = SF.iso_target_size(mesh.coords, mesh.tets, err, target)
            assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
