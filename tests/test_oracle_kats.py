"""Pin the CPU oracle against the reference's own known-answer tests.

Every expected vector comes from tests/golden/reference_kats.json, parsed
verbatim from the rustpde sources (file:line recorded there).  The inputs are
rebuilt here exactly as the cited reference test builds them.  The reference
asserts |diff| <= 1e-3; the oracle is held to the printed precision of each
vector (exact vectors: 1e-12).
"""
import numpy as np
import pytest

from oracle import oracle as O


def kv(kats, name):
    return np.array(kats[name]["values"], dtype=np.float64)


def close(got, exp, atol):
    got = np.asarray(got)
    exp = np.asarray(exp)
    assert got.shape == exp.shape, (got.shape, exp.shape)
    err = np.max(np.abs(got - exp)) if got.size else 0.0
    assert err <= atol, f"max abs diff {err:.3e} > {atol:.1e}"


def flat_index(shape):
    return np.arange(np.prod(shape), dtype=np.float64).reshape(shape)


# ---------------------------------------------------------------- Chebyshev
def test_cheb_forward_backward_doctest(kats):
    # funspace/src/chebyshev/ortho.rs:210-221, 260-271
    x = np.array([1.0, 2.0, 3.0, 4.0])
    close(O.base_forward(O.CHEB, 4, x), [2.5, 4.0 / 3.0, 0.0, 1.0 / 6.0], 1e-14)
    close(O.base_forward(O.CHEB, 4, x), kv(kats, "cheb_forward_4"), 1e-8)
    close(O.base_backward(O.CHEB, 4, x), kv(kats, "cheb_backward_4"), 1e-13)


def test_cheb_differentiate_lane_doctest(kats):
    # ortho.rs:90-105
    x = np.array([1.0, 2.0, 3.0, 4.0])
    close(O.base_differentiate(O.CHEB, 4, x, 2), kv(kats, "cheb_diff_lane_twice"), 1e-12)
    close(O.base_differentiate(O.CHEB, 4, x, 0), kv(kats, "cheb_diff_lane_zero"), 0.0)


def test_cheb_differentiate_2d(kats):
    # ortho.rs:626-664 (data[i] = flat index, 6x4)
    data = flat_index((6, 4))
    sp = O.Space2(O.CHEB, 6, O.CHEB, 4)
    close(sp.gradient(data, (1, 0)), kv(kats, "cheb_differentiate_axis0"), 1e-11)
    close(sp.gradient(data, (0, 1)), kv(kats, "cheb_differentiate_axis1"), 1e-11)


def test_pinv_identity_doctest():
    # ortho.rs:495-506: (pinv . lap)[2:, :] == laplace_inv_eye
    lap = O.base_matrix(O.CHEB, 5, 1)
    pinv = O.base_matrix(O.CHEB, 5, 2)
    eye = O.base_matrix(O.CHEB, 5, 3)
    close((pinv @ lap)[2:, :], eye, 1e-14)


def test_nodes_gauss_lobatto():
    # ortho.rs:71-80: x_k = -sin(pi (m - 2k) / (2m)), ascending -1 .. 1
    x = O.base_coords(O.CHEB, 9)
    close(x, -np.cos(np.pi * np.arange(9) / 8), 1e-15)


# ---------------------------------------------------------------- composite
def test_cd_to_from_ortho_doctests(kats):
    # composite.rs:122-143 and 183-202 (nx, ny) = (5, 4)
    sp = O.Space2(O.CD, 5, O.CHEB, 4)
    close(sp.to_ortho(flat_index((3, 4))), kv(kats, "cd_to_ortho_doc"), 1e-13)
    close(sp.from_ortho(flat_index((5, 4))), kv(kats, "cd_from_ortho_doc"), 1e-12)


def test_cd_to_ortho_unit(kats):
    # composite.rs:611-647
    close(O.Space2(O.CD, 5, O.CHEB, 4).to_ortho(flat_index((3, 4))), kv(kats, "cd_to_ortho_axis0"), 1e-13)
    close(O.Space2(O.CHEB, 5, O.CD, 4).to_ortho(flat_index((5, 2))), kv(kats, "cd_to_ortho_axis1"), 1e-13)


def test_cd_differentiate_unit(kats):
    # composite.rs:649-688: ChebDirichlet(n+2), twice, data (6, 4) flat index
    data = flat_index((6, 4))
    close(O.Space2(O.CD, 8, O.CHEB, 4).gradient(data, (2, 0)), kv(kats, "cd_differentiate_axis0"), 1e-9)
    close(O.Space2(O.CHEB, 6, O.CD, 6).gradient(data, (0, 2)), kv(kats, "cd_differentiate_axis1"), 1e-9)


def test_cd_forward_backward_differentiate_doctests(kats):
    # composite.rs:353-362, 398-409, 513-522
    close(O.base_forward(O.CD, 5, [1.0, 2.0, 3.0, 4.0, 5.0]), [2.0, np.sqrt(0.5), 1.0], 1e-14)
    close(O.base_forward(O.CD, 5, [1.0, 2.0, 3.0, 4.0, 5.0]), kv(kats, "cd_forward_5"), 1e-8)
    close(O.base_backward(O.CD, 5, [1.0, 2.0, 3.0]), kv(kats, "cd_backward_5"), 1e-4)
    close(O.base_backward(O.CD, 5, [1.0, 2.0, 3.0]), [0.0, 4 - 2 * np.sqrt(2), -4.0, 4 + 2 * np.sqrt(2), 0.0], 1e-13)
    close(O.base_differentiate(O.CD, 5, [1.0, 2.0, 3.0], 2), kv(kats, "cd_differentiate_5"), 1e-12)


def test_stencils(kats):
    # composite_stencil.rs:415-454
    close(O.base_from_ortho(O.CD, 5, kv(kats, "stencil_parent_in")), kv(kats, "stencil_composite_out"), 1e-4)
    close(O.base_to_ortho(O.CD, 5, kv(kats, "stencil_composite_in")), kv(kats, "stencil_parent_out"), 1e-4)
    close(O.base_from_ortho(O.CDBC, 4, kv(kats, "stencil_bc_parent_in")), kv(kats, "stencil_bc_composite_out"), 1e-14)
    close(O.base_to_ortho(O.CDBC, 4, kv(kats, "stencil_bc_composite_in")), kv(kats, "stencil_bc_parent_out"), 1e-14)


def test_stencil_complex():
    # composite_stencil.rs:428-441: complex data (x, x) behaves like (1+i) * real
    sp = O.Space2(O.FOURIER, 4, O.CD, 5)  # complex spectral space, CD along axis 1
    parent = np.array([2.0, 0.7071, -1.0, -0.7071, -1.0])
    p2 = np.tile(parent * (1 + 1j), (3, 1))
    c2 = sp.from_ortho(p2)
    close(c2.real, np.tile(O.base_from_ortho(O.CD, 5, parent), (3, 1)), 1e-14)
    close(c2.imag, c2.real, 0.0)


# ---------------------------------------------------------------- Fourier
def test_fourier_doctests(kats):
    # r2c.rs:130-147, 177-194
    f = O.base_forward(O.FOURIER, 4, [1.0, 2.0, 3.0, 4.0])
    exp = kv(kats, "fourier_forward_4")
    close(np.stack([f.real, f.imag], axis=1), exp, 1e-14)
    back = O.base_backward(O.FOURIER, 4, exp[:, 0] + 1j * exp[:, 1])
    close(back, kv(kats, "fourier_backward_4"), 1e-14)


def test_fourier_derivative_accuracy():
    # funspace/src/lib.rs:45-72: d2/dx2 sin(2x) on 8 points, |err| < 1e-5
    x = O.base_coords(O.FOURIER, 8)
    vh = O.base_forward(O.FOURIER, 8, np.sin(2 * x))
    dvh = O.base_differentiate(O.FOURIER, 8, vh, 2)
    dv = O.base_backward(O.FOURIER, 8, dvh)
    close(dv, -4 * np.sin(2 * x), 1e-12)


def test_fourier_c2r_ignores_dc_nyquist_imag():
    rng = np.random.default_rng(0)
    xh = rng.standard_normal(5) + 1j * rng.standard_normal(5)
    a = O.base_backward(O.FOURIER, 8, xh)
    xh2 = xh.copy()
    xh2[0] = xh2[0].real
    xh2[4] = xh2[4].real
    close(a, O.base_backward(O.FOURIER, 8, xh2), 0.0)
    close(a, np.fft.irfft(xh, 8), 1e-15)


# ---------------------------------------------------------------- averages
def test_average_doctests():
    # src/field/average.rs:11-24, 36-50
    sp = O.Space2(O.CHEB, 6, O.CHEB, 5)
    v = np.tile(np.arange(5.0), (6, 1))
    close(sp.average_axis(v, 0), [0.0, 1.0, 2.0, 3.0, 4.0], 1e-15)
    assert abs(sp.average(v) - 2.0) < 1e-15


# ---------------------------------------------------------------- solvers
def test_hholtz_adi_1d(kats):
    # src/solver/hholtz_adi.rs:153-173 (pypde values, 8 decimals)
    x = O.solver1d(O.CD, 7, O.HHOLTZ_ADI, 1.0, np.arange(1.0, 8.0))
    close(x, kv(kats, "hholtz_adi_1d"), 1e-8)


def test_hholtz_adi_2d(kats):
    # hholtz_adi.rs:175-207 (4 significant digits)
    sp = O.Space2(O.CD, 7, O.CD, 7)
    b = np.tile(np.arange(1.0, 8.0), (7, 1))
    x = O.Solver(sp, O.HHOLTZ_ADI, (1.0, 1.0)).solve(b)
    exp = kv(kats, "hholtz_adi_2d")
    assert np.all(np.abs(x - exp) <= 5.1e-4 * np.abs(exp) + 1e-12)


def test_poisson_1d(kats):
    # src/solver/poisson.rs:187-205 (4 decimals, truncated: one unit of the last digit)
    x = O.solver1d(O.CD, 8, O.POISSON, 1.0, np.arange(1.0, 9.0))
    close(x, kv(kats, "poisson_1d"), 1.0001e-4)
    # the same solution in closed form (rationals), which the printed digits truncate
    close(x, [5 / 48, 17 / 210, 1 / 16, 11 / 280, -1 / 24, -1 / 28], 1e-15)


def test_poisson_2d(kats):
    # poisson.rs:207-240 (6-8 decimals)
    sp = O.Space2(O.CD, 8, O.CD, 7)
    b = np.tile(np.arange(1.0, 8.0), (8, 1))
    x = O.Solver(sp, O.POISSON, (1.0, 1.0)).solve(b)
    close(x, kv(kats, "poisson_2d"), 1e-6)


def test_poisson_2d_complex(kats):
    # poisson.rs:241-274: b = (x, x) -> y (1 + i)
    sp = O.Space2(O.FOURIER, 16, O.CD, 7)  # only to obtain a complex oracle space
    b = np.tile(np.arange(1.0, 8.0), (8, 1))
    spr = O.Space2(O.CD, 8, O.CD, 7)
    x_re = O.Solver(spr, O.POISSON, (1.0, 1.0)).solve(b)
    exp = kv(kats, "poisson_2d_complex")
    close(x_re, exp, 1e-6)  # the real and imaginary parts are solved independently
    del sp


def test_tensor2d_recovery(kats):
    # src/solver/fdma_tensor.rs:321-356
    a = kv(kats, "tensor2d_a")
    c = kv(kats, "tensor2d_c")
    data = flat_index((6, 6))
    x = O.Tensor2(a, c, 0.0).solve(data)
    rec = a @ x @ c.T + c @ x @ a.T
    close(rec, data, 1e-9)


def _test_matrix(nx):
    # fdma.rs:262-288 / matvec.rs:329-359 test matrix
    m = np.zeros((nx, nx))
    for i in range(nx):
        j = i + 1.0
        m[i, i] = 0.5 * j
        if i > 1:
            m[i, i - 2] = 10.0 * j
        if i < nx - 2:
            m[i, i + 2] = 1.5 * j
        if i < nx - 4:
            m[i, i + 4] = 2.5 * j
    return m


def test_fdma_recovery():
    mat = _test_matrix(6)
    b = np.arange(6.0)
    x = O.fdma_solve(mat, b)
    close(mat @ x, b, 1e-12)
    bc = np.arange(6.0) + 1j * np.arange(1.0, 7.0)
    xc = O.fdma_solve(mat, bc)
    close(mat @ xc, bc, 1e-12)


def test_matvec_fdma():
    # matvec.rs:329-359: (nx, nx+2) banded matrix against (nx+2, nx+2) data
    nx = 6
    full = _test_matrix(nx + 2)[:nx, :]
    m = np.zeros((nx, nx + 2))
    for i in range(nx):
        j = i + 1.0
        m[i, i] = 0.5 * j
        if i > 1:
            m[i, i - 2] = 10.0 * j
        if i < nx - 2:
            m[i, i + 2] = 1.5 * j
        if i < nx - 4:
            m[i, i + 4] = 2.5 * j
    del full
    data = flat_index((nx + 2, nx + 2))
    close(O.matvec_fdma(m, data, 0), m @ data, 1e-12)
    close(O.matvec_fdma(m, data, 1), (m @ data.T).T, 1e-12)


def test_eig_reconstruction():
    # src/solver/utils.rs:181-202 through the same numpy/LAPACK path the oracle uses
    t = np.tile(np.arange(1.0, 6.0), (5, 1))
    lam, fwd, bwd = O.tensor_eig(t, np.eye(5))
    close(bwd @ np.diag(lam) @ fwd, t, 1e-12)
    assert np.all(np.diff(lam) <= 0)


# ---------------------------------------------------------------- analytic
def _grid_field(sp):
    (x, y), _ = sp.coords()
    return x, y


@pytest.mark.parametrize("kind,c,nx,ny", [
    (O.HHOLTZ, (1.0, 1.0), 64, 64),       # hholtz.rs:219-249
    (O.HHOLTZ_ADI, (1e-5, 1e-5), 16, 7),  # hholtz_adi.rs:209-239
])
def test_hholtz_cd_cd_analytic(kind, c, nx, ny):
    sp = O.Space2(O.CD, nx, O.CD, ny)
    x, y = _grid_field(sp)
    n = np.pi / 2
    v = np.cos(n * x)[:, None] * np.cos(n * y)[None, :]
    alpha = c[0]
    exp = 1.0 / (1.0 + alpha * n * n * 2.0) * v
    vh = sp.forward(v)
    out = O.Solver(sp, kind, c).solve(sp.to_ortho(vh))
    close(sp.backward(out), exp, 1e-3 if kind == O.HHOLTZ_ADI else 1e-6)


@pytest.mark.parametrize("kind", [O.HHOLTZ, O.HHOLTZ_ADI])
def test_hholtz_fo_cd_analytic(kind):
    # hholtz.rs:251-279, hholtz_adi.rs:241-269
    sp = O.Space2(O.FOURIER, 16, O.CD, 7)
    x, y = _grid_field(sp)
    n = np.pi / 2
    alpha = 1e-5
    v = np.cos(x)[:, None] * np.cos(n * y)[None, :]
    exp = 1.0 / (1.0 + alpha * n * n + alpha) * v
    out = O.Solver(sp, kind, (alpha, alpha)).solve(sp.to_ortho(sp.forward(v)))
    close(sp.backward(out), exp, 1e-3)


def test_poisson_cd_cd_analytic():
    # poisson.rs:276-307
    sp = O.Space2(O.CD, 8, O.CD, 7)
    x, y = _grid_field(sp)
    n = np.pi / 2
    v = np.cos(n * x)[:, None] * np.cos(n * y)[None, :]
    exp = -1.0 / (n * n * 2.0) * v
    out = O.Solver(sp, O.POISSON, (1.0, 1.0)).solve(sp.to_ortho(sp.forward(v)))
    close(sp.backward(out), exp, 1e-3)


def test_poisson_fo_cd_analytic():
    # poisson.rs:309-339
    sp = O.Space2(O.FOURIER, 16, O.CD, 7)
    x, y = _grid_field(sp)
    ny_, nx_ = np.pi / 2, 2.0
    v = np.cos(nx_ * x)[:, None] * np.cos(ny_ * y)[None, :]
    exp = -1.0 / (nx_ * nx_ + ny_ * ny_) * v
    out = O.Solver(sp, O.POISSON, (1.0, 1.0)).solve(sp.to_ortho(sp.forward(v)))
    close(sp.backward(out), exp, 1e-3)


def test_conv_term_analytic():
    # src/navier/conv_term.rs:64-119 : u * dT/dx and u * dT/dy on 12x12
    n = 12
    tsp = O.Space2(O.CD, n, O.CN, n)
    fsp = O.Space2(O.CHEB, n, O.CHEB, n)
    (x, y), _ = fsp.coords()
    ax, ay = np.pi, np.pi
    temp = np.sin(ax * x)[:, None] * np.cos(ay * y)[None, :]
    ux = np.sin(ax * x)[:, None] * np.sin(ay * y)[None, :]
    th = tsp.forward(temp)
    for deriv, exact in (((1, 0), ax * np.cos(ax * x)[:, None] * np.cos(ay * y)[None, :]),
                         ((0, 1), np.sin(ax * x)[:, None] * -ay * np.sin(ay * y)[None, :])):
        conv = ux * fsp.backward(tsp.gradient(th, deriv))
        close(conv, exact * ux, 1e-3)


@pytest.mark.parametrize("n", [4, 17, 33, 64, 129])
def test_dense_dct_switch_is_the_same_transform(n):
    # or_set_dense_dct: DCT-I of length n by its defining sum instead of the
    # FFT; the two agree to rounding (the switch only measures a case's
    # sensitivity to the transform's rounding)
    x = np.random.default_rng(n).standard_normal(n)
    ref = O.base_forward(O.CHEB, n, x)
    refb = O.base_backward(O.CHEB, n, x)
    O.set_dense_dct(n)
    try:
        d = O.base_forward(O.CHEB, n, x)
        db = O.base_backward(O.CHEB, n, x)
    finally:
        O.set_dense_dct(-1)
    close(d, ref, 1e-13 * np.max(np.abs(ref)))
    close(db, refb, 1e-13 * np.max(np.abs(refb)))
    assert np.array_equal(O.base_forward(O.CHEB, n, x), ref)
