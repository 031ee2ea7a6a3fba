"""Navier2DAdjoint (src/navier/navier_adjoint.rs) on the GPU against the CPU
FP64 oracle's restatement, same initial fields.

Tolerances: relative L2 per field <= 1e-9 after 10 adjoint updates (each
update is a Navier2D step, three Helmholtz smoothings, eleven convection
products and a projection; the device commutes axis passes), diagnostics and
residual norms <= 1e-9 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

STATE = (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1)
RES = (O.TEMP_RES, O.UX_RES, O.UY_RES)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


CASES = {
    "box32": (32, 32, 1e4, 1.0, 0.02, 1.0, O.BOX_ADIABATIC),
    "box_cond33_asp15": (33, 33, 3e4, 0.7, 0.01, 1.5, O.BOX_CONDUCTING),
    "periodic64x33": (64, 33, 1e4, 1.0, 0.02, 1.0, O.PERIODIC),
}


def pair(R, name):
    args = CASES[name]
    o = O.Navier2DAdjoint(*args)
    g = R.Navier2DAdjoint(*args)
    for a in (o, g):
        a.set_temperature(0.5, 1.0, 1.0)
        a.set_velocity(0.5, 1.0, 1.0)
    return o, g


@pytest.mark.parametrize("name", list(CASES))
def test_initial_fields(R, name):
    o, g = pair(R, name)
    for f in (O.TEMP, O.UX, O.UY):
        assert rel(g.get(f), o.get(f)) < 1e-13


@pytest.mark.parametrize("name", list(CASES))
def test_ten_updates(R, name):
    o, g = pair(R, name)
    o.update(10)
    g.update(10)
    for f in STATE + RES:
        e = rel(g.get(f), o.get(f))
        assert e < 1e-9, (name, f, e)
    assert abs(g.get_time() - o.time) < 1e-12
    ro, rg = o.residual(), g.residual()
    np.testing.assert_allclose(rg, ro, rtol=1e-9)


@pytest.mark.parametrize("name", ["box32", "periodic64x33"])
def test_diagnostics_and_exit(R, name):
    o, g = pair(R, name)
    o.update(5)
    g.update(5)
    for what in (O.NU, O.NUVOL, O.RE, O.KE, O.DIVNORM):
        a, b = g.eval(what), o.eval(what)
        assert abs(a - b) <= 1e-9 * abs(b) + 1e-13, (what, a, b)
    assert g.exit() is False and o.exit() is False


def test_descent_reduces_the_residual(R):
    """The smoothed residual falls along the descent (navier_adjoint.rs)."""
    _, g = pair(R, "box32")
    g.update(5)
    r0 = g.residual()[3:].sum()
    g.update(60)
    r1 = g.residual()[3:].sum()
    assert r1 < 0.8 * r0, (r0, r1)


def test_integrate_and_callback(R):
    _, g = pair(R, "periodic64x33")
    seen = []
    n = R.integrate(g, 0.2, 0.1, callback=lambda a: seen.append(a.callback()))
    assert n == 10
    assert len(seen) == 2
    assert all(np.isfinite(d["Nu"]) and d["res_smoothed"] > 0 for d in seen)


def test_state_round_trip_and_errors(R):
    _, g = pair(R, "box32")
    t = g.get(O.TEMP)
    g.set(O.TEMP, 2 * t)
    np.testing.assert_array_equal(g.get(O.TEMP), 2 * t)
    with pytest.raises(ValueError):
        g.set(O.TEMP, np.zeros((3, 3)))
    with pytest.raises(R.RbcError):
        R.Navier2DAdjoint(32, 32, -1.0, 1.0, 0.02, 1.0, O.BOX_ADIABATIC)


def test_snapshot_write_read(R, tmp_path):
    """write() stores the adjoint state; read() restores temp, ux, uy and time."""
    from rustpde_gb300.snapshot import read_snapshot
    _, g = pair(R, "box32")
    g.update(3)
    path = str(tmp_path / "adjoint.rbc")
    g.write(path)
    snap = read_snapshot(path)
    np.testing.assert_array_equal(snap["datasets"]["ux/vhat"], g.get(O.UX))
    assert abs(snap["scalars"]["time"] - g.get_time()) < 1e-15
    h = R.Navier2DAdjoint(*CASES["box32"])
    h.read(path)
    for f in (O.TEMP, O.UX, O.UY):
        np.testing.assert_array_equal(h.get(f), g.get(f))
    assert abs(h.get_time() - g.get_time()) < 1e-15
