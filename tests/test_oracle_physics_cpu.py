"""Physical properties of the oracle's full Navier2D step (CPU), beside the
component known-answer tests that pin it: a fluid at rest stays (nearly) at
rest, and below the onset of convection a perturbation decays."""
import numpy as np
import pytest

from oracle import oracle as O

KINDS = [O.BOX_ADIABATIC, O.BOX_CONDUCTING, O.PERIODIC]


def case(kind, ra, dt=0.01):
    nx, ny = (32, 33) if kind == O.PERIODIC else (24, 24)
    return O.Navier2D(nx, ny, ra, 1.0, dt, 1.0, kind)


@pytest.mark.parametrize("kind", KINDS)
def test_rest_state_stays_at_rest(kind):
    # zero velocity, temperature deviation and pressure on top of the
    # conduction profile (the boundary field): the buoyancy is balanced by a
    # hydrostatic pressure that the steps build up; the velocity stays at the
    # level of the pressure-projection splitting error
    n = case(kind, 1e4)
    for f in (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1):
        sh, _, cx = n.shape(f)
        n.set(f, np.zeros(sh, dtype=np.complex128 if cx else np.float64))
    n.update(20)
    ke = n.eval_ke()
    assert ke < (1e-25 if kind == O.PERIODIC else 1e-7), ke
    assert abs(n.eval_nu() - n.eval_nuvol()) < 1e-4 * abs(n.eval_nuvol())


@pytest.mark.parametrize("kind", KINDS)
def test_subcritical_perturbation_decays(kind):
    # Ra = 500 is below the onset of convection for every wall type here:
    # the kinetic energy of a small perturbation falls monotonically
    n = case(kind, 500.0)
    O.standard_ic(n, 3, vel_amp=1e-2)
    kes = []
    for _ in range(6):
        n.update(20)
        kes.append(n.eval_ke())
    assert all(b < a for a, b in zip(kes, kes[1:])), kes
    assert kes[-1] < 0.2 * kes[0], kes
