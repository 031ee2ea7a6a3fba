"""The oracle's Navier2DAdjoint (src/navier/navier_adjoint.rs): properties of
the descent that hold without the GPU.  The reference has no test for this
solver; its GPU form is compared with this restatement in test_gpu_adjoint.py.
"""
import numpy as np

from oracle import oracle as O


def test_smoothed_residual_decreases():
    a = O.Navier2DAdjoint(24, 24, 1e4, 1.0, 0.02, 1.0, O.BOX_ADIABATIC)
    a.set_temperature(0.5, 1.0, 1.0)
    a.set_velocity(0.5, 1.0, 1.0)
    a.update(3)
    r0 = a.residual()[3:].sum()
    a.update(40)
    r1 = a.residual()[3:].sum()
    assert r1 < 0.8 * r0
    assert not a.exit()


def test_conduction_state_is_nearly_steady():
    """The conduction state (no perturbation; the boundary field carries the
    linear temperature profile) is steady: the buoyancy is a pure gradient
    that the projection removes.  With periodic sidewalls the residuals stay
    at rounding level; in the box the Chebyshev-tau projection leaves a small
    remainder."""
    a = O.Navier2DAdjoint(16, 17, 1e4, 1.0, 0.02, 1.0, O.PERIODIC)
    a.update(2)
    for f in (O.TEMP_RES, O.UX_RES, O.UY_RES):
        assert np.abs(a.get(f)).max() < 1e-13, f
    b = O.Navier2DAdjoint(16, 16, 1e4, 1.0, 0.02, 1.0, O.BOX_ADIABATIC)
    b.update(2)
    for f in (O.TEMP_RES, O.UX_RES, O.UY_RES):
        assert np.abs(b.get(f)).max() < 1e-3, f


def test_time_advances_by_dt():
    a = O.Navier2DAdjoint(16, 16, 1e4, 1.0, 0.05, 1.0, O.BOX_CONDUCTING)
    a.update(4)
    assert abs(a.time - 0.2) < 1e-12
