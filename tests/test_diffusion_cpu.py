"""The oracle's Diffusion2D (src/navier/diffusion.rs:113-238) against the
mathematics it discretises: one implicit Euler step of u_t = kappa lap u with
the Helmholtz operator (I - dt kappa D2x - dt kappa D2y) (hholtz.rs:42-76,
alpha = 1) scales an eigenfunction of the Laplacian by 1 / (1 + dt kappa lam).
Spectral accuracy: 1e-10 at 33 x 33.
"""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("kappa,dt", [(1.0, 0.01), (0.3, 0.05)])
def test_eigenmode_decay_dirichlet(kappa, dt):
    d = O.Diffusion2D(O.CD, 33, O.CD, 33, kappa, dt)
    (x, y), _ = d.space.coords()
    u0 = np.cos(np.pi * x / 2)[:, None] * np.cos(np.pi * y / 2)[None, :]
    d.vhat = d.space.forward(u0)
    d.update(1)
    lam = 2 * (np.pi / 2) ** 2
    np.testing.assert_allclose(d.physical(), u0 / (1 + dt * kappa * lam), atol=1e-10)


def test_eigenmode_decay_fourier_dirichlet():
    kappa, dt = 0.5, 0.02
    d = O.Diffusion2D(O.FOURIER, 32, O.CD, 33, kappa, dt)
    (x, y), _ = d.space.coords()
    u0 = np.sin(3 * x)[:, None] * np.cos(np.pi * y / 2)[None, :]
    d.vhat = d.space.forward(u0)
    d.update(1)
    lam = 9 + (np.pi / 2) ** 2
    np.testing.assert_allclose(d.physical(), u0 / (1 + dt * kappa * lam), atol=1e-10)


def test_steady_state_with_force():
    """-kappa lap u = f has the steady state of the forced iteration: with
    f = kappa lam phi for the eigenfunction phi, u -> phi."""
    kappa, dt = 1.0, 0.5
    d = O.Diffusion2D(O.CD, 33, O.CD, 33, kappa, dt)
    (x, y), _ = d.space.coords()
    phi = np.cos(np.pi * x / 2)[:, None] * np.cos(np.pi * y / 2)[None, :]
    lam = 2 * (np.pi / 2) ** 2
    # the force is added to the ortho-space right-hand side: its Chebyshev coefficients
    fsp = O.Space2(O.CHEB, 33, O.CHEB, 33)
    d.add_force(fsp.forward(kappa * lam * phi))
    d.update(200)
    np.testing.assert_allclose(d.physical(), phi, atol=1e-9)
