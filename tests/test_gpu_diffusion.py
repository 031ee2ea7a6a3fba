"""Diffusion2D (src/navier/diffusion.rs:113-238) on the GPU against the CPU
FP64 oracle on the same inputs.

Tolerance: relative L2 of the spectral state <= 1e-11 after 20 steps (each
step is one Helmholtz solve of a linear problem; the device reassociates the
constant term and the axis order of the commuting operators).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


SPACES = {
    "cd33xcd33": (O.CD, 33, O.CD, 33),
    "cd48xcn40": (O.CD, 48, O.CN, 40),
    "cn65xcd64": (O.CN, 65, O.CD, 64),
    "fourier64xcd33": (O.FOURIER, 64, O.CD, 33),
    "fourier128xcn65": (O.FOURIER, 128, O.CN, 65),
    "fourier96xcd33": (O.FOURIER, 96, O.CD, 33),
}


def pair(R, name, kappa=1.0, dt=0.01):
    k0, n0, k1, n1 = SPACES[name]
    o = O.Diffusion2D(k0, n0, k1, n1, kappa, dt)
    field = R.Field2(R.Space2(R.Base(k0, n0), R.Base(k1, n1)))
    g = R.Diffusion2D(field, kappa, dt)
    return o, g


@pytest.mark.parametrize("name", list(SPACES))
def test_impulse_then_steps(R, name):
    o, g = pair(R, name)
    o.impulse()
    g.impulse()
    assert rel(g.get_state(), o.vhat) < 1e-13
    o.update(20)
    g.update(20)
    e = rel(g.get_state(), o.vhat)
    assert e < 1e-11, (name, e)
    assert abs(g.get_time() - o.time) < 1e-12
    assert rel(g.get_physical(), o.physical()) < 1e-11


@pytest.mark.parametrize("name", ["cd33xcd33", "cn65xcd64"])
def test_force(R, name):
    o, g = pair(R, name, kappa=0.5, dt=0.02)
    n0, n1 = SPACES[name][1], SPACES[name][3]
    rng = np.random.default_rng(11)
    f = rng.standard_normal((n0, n1))
    o.add_force(f)
    g.add_force(f)
    o.impulse()
    g.impulse()
    o.update(15)
    g.update(15)
    assert rel(g.get_state(), o.vhat) < 1e-11


def test_force_rejected_on_fourier(R):
    _, g = pair(R, "fourier64xcd33")
    with pytest.raises(R.RbcError):
        g.add_force(np.zeros((64, 33)))


@pytest.mark.parametrize("name,bc", [("cd33xcd33", (O.CHEB, O.CDBC)), ("fourier64xcd33", (O.FOURIER, O.CDBC))])
def test_fieldbc(R, name, bc):
    """An inhomogeneous boundary field: T = +-0.5 at the plates (bc_rbc)."""
    o, g = pair(R, name, kappa=0.2, dt=0.01)
    k0, n0, k1, n1 = SPACES[name]
    sp = O.Space2(bc[0], n0, bc[1], n1)
    # a smooth profile carried by the two boundary modes
    bvh = sp._spec_arr(sp.spec)
    for i in range(sp.spec[0]):
        bvh[i, 0] = 0.5 / (1 + i)
        bvh[i, 1] = -0.25 / (1 + i)
    o.add_fieldbc(bc[0], bc[1], bvh)
    fbc = R.Field2(R.Space2(R.Base(bc[0], n0), R.Base(bc[1], n1)))
    fbc.vhat = bvh
    g.add_fieldbc(fbc)
    o.impulse()
    g.impulse()
    o.update(10)
    g.update(10)
    assert rel(g.get_state(), o.vhat) < 1e-11
    assert rel(g.callback(), o.physical(with_bc=True)) < 1e-11


def test_integrate_loop(R):
    """integrate() (lib.rs:155-187) drives a Diffusion2D to max_time."""
    o, g = pair(R, "cd33xcd33", dt=0.01)
    g.impulse()
    o.impulse()
    saved = []
    n = R.integrate(g, 0.2, 0.05, callback=lambda p: saved.append(p.get_time()))
    o.update(n)
    assert n == 20
    assert len(saved) == 4
    assert rel(g.get_state(), o.vhat) < 1e-11


def test_decay_is_monotone(R):
    """Pure diffusion with homogeneous walls: the L2 norm of the physical
    field decreases step by step."""
    _, g = pair(R, "cd48xcn40", kappa=1.0, dt=1e-3)
    g.impulse()
    prev = np.linalg.norm(g.get_physical())
    for _ in range(5):
        g.update(1)
        cur = np.linalg.norm(g.get_physical())
        assert cur < prev
        prev = cur
