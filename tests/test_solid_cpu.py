"""Solid masks on the CPU: the library's host mask generators
(src/navier/solid_masks.rs, exported as rbc_solid_*) against the oracle's
numpy restatement, and the oracle's penalisation branch (navier.rs:551-608).

The reference has no known-answer test for solid masks; the generators are
pinned against the restatement at 1e-14 absolute (the two use different
tanh/pow implementations), the Navier2D branch against the GPU path in
test_gpu_solid.py.
"""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def S():
    from rustpde_gb300 import build
    build.build()
    from rustpde_gb300 import solid_masks
    return solid_masks


def cheb_nodes(n):
    return -np.cos(np.pi * np.arange(n) / (n - 1))


GRIDS = {
    "cheb33x33": (cheb_nodes(33), cheb_nodes(33)),
    "scaled65x33": (1.7 * cheb_nodes(65), cheb_nodes(33)),
    "fourier64x17": (np.arange(64) * 2 * np.pi / 64, cheb_nodes(17)),
    "ragged5x3": (np.array([-1.0, -0.3, 0.0, 0.4, 1.0]), np.array([-1.0, 0.1, 1.0])),
}


@pytest.mark.parametrize("grid", list(GRIDS))
@pytest.mark.parametrize("args", [(0.2, 0.0, 0.2), (0.0, 0.0, 0.5), (-0.5, 0.3, 0.05), (3.0, 3.0, 0.1)])
def test_cylinder_inner(S, grid, args):
    x, y = GRIDS[grid]
    a, b = S.solid_cylinder_inner(x, y, *args), O.solid_cylinder_inner(x, y, *args)
    assert a[0].shape == (x.size, y.size)
    np.testing.assert_allclose(a[0], b[0], rtol=0, atol=1e-14)
    assert np.all(a[1] == 0)
    assert a[0].min() >= 0.0 and a[0].max() <= 1.0


@pytest.mark.parametrize("grid", list(GRIDS))
@pytest.mark.parametrize("args", [(0.1, 6.0), (0.05, 2.0), (0.6, 1.0)])
def test_roughness_sinusoid(S, grid, args):
    x, y = GRIDS[grid]
    a, b = S.solid_roughness_sinusoid(x, y, *args), O.solid_roughness_sinusoid(x, y, *args)
    np.testing.assert_allclose(a[0], b[0], rtol=0, atol=1e-14)
    np.testing.assert_array_equal(a[1], b[1])
    assert set(np.unique(a[1])) <= {-0.5, 0.0, 0.5}


@pytest.mark.parametrize("grid", ["cheb33x33", "scaled65x33"])
@pytest.mark.parametrize("args", [(0.3, 0.6), (0.2, 0.9), (0.5, 0.0), (0.4, 1.0)])
def test_porosity(S, grid, args):
    x, y = GRIDS[grid]
    a, b = S.solid_porosity(x, y, *args), O.solid_porosity(x, y, *args)
    np.testing.assert_allclose(a[0], b[0], rtol=0, atol=1e-13)
    assert np.all(a[1] == 0)


def test_generator_errors(S):
    import rustpde_gb300 as R
    x = cheb_nodes(9)
    with pytest.raises(R.RbcError):
        S.solid_cylinder_inner(x, x, 0.0, 0.0, -1.0)
    with pytest.raises(R.RbcError):
        S.solid_porosity(x, x, 0.2, 1.5)


@pytest.mark.parametrize("kind", [O.BOX_ADIABATIC, O.PERIODIC])
def test_oracle_zero_mask_is_no_solid(kind):
    """A zero mask leaves the oracle's step bit-identical (damping term 0)."""
    a = O.Navier2D(16, 17, 1e5, 1.0, 0.01, 1.0, kind)
    b = O.Navier2D(16, 17, 1e5, 1.0, 0.01, 1.0, kind)
    for n in (a, b):
        O.standard_ic(n, 5)
    a.set_solid(np.zeros((16, 17)), np.zeros((16, 17)))
    a.update(3)
    b.update(3)
    for f in (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1):
        np.testing.assert_array_equal(a.get(f), b.get(f))


def test_oracle_solid_damps_velocity():
    """Inside a full-strength obstacle the velocity decays relative to the
    free flow (the Brinkman term acts as a drag of rate 1/eta)."""
    a = O.Navier2D(24, 24, 1e4, 1.0, 0.005, 1.0, O.BOX_ADIABATIC)
    b = O.Navier2D(24, 24, 1e4, 1.0, 0.005, 1.0, O.BOX_ADIABATIC)
    for n in (a, b):
        O.standard_ic(n, 2, vel_amp=0.5)
    x, y = a.coords(O.TEMP)
    m, v = O.solid_cylinder_inner(x, y, 0.0, 0.0, 0.5)
    a.set_solid(m, v)
    a.update(20)
    b.update(20)
    inside = m > 0.99
    ua, ub = a.get_phys(O.UX), b.get_phys(O.UX)
    assert np.abs(ua[inside]).max() < 0.5 * np.abs(ub[inside]).max()
