"""Sizes at the edges of what the kernels run.

* The smallest grids (8 x 8, box and periodic) against the oracle.
* The reference's largest benchmark box, 513 x 513 (benches/benchmark_navier.rs).
  A CTA pass keeps the lanes it transforms in shared memory. A Chebyshev
  transform through an FFT needs 2(n - 1) more complex work elements per lane,
  which the box x pass cannot hold at this size, so that axis uses the dense
  transform. At this size rounding alone moves the results by more than
  1e-10; the tolerance is 4x the spread the oracle itself shows between two
  exact restatements of its transform and of its eigen-decomposition.
* The reference's smooth initial fields (set_velocity, set_temperature)
  against the oracle, at the usual 1e-10.
* Sizes whose passes fit a block's shared memory in no form are refused at
  creation with RBC_ERR_INVALID, not at the first step. Where the mixed form's
  passes still fit, it runs.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FIELDS = (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def pair(R, kind, nx, ny, ra, pr, dt, asp, precision=None, seed=1):
    o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
    O.standard_ic(o, seed)
    g = R.Navier2D(nx, ny, ra, pr, dt, asp, kind, precision=precision or R.PREC_FP64, seed=None)
    R.standard_ic(g, seed)
    return o, g


SMALL = {
    "box8": (O.BOX_ADIABATIC, 8, 8, 1e4, 1.0, 1e-2, 1.0),
    "box_cond8": (O.BOX_CONDUCTING, 8, 8, 1e4, 0.7, 1e-2, 1.5),
    "periodic8": (O.PERIODIC, 8, 8, 1e4, 1.0, 1e-2, 1.0),
}


@pytest.mark.parametrize("name", list(SMALL))
def test_smallest_grids(R, name):
    o, g = pair(R, *SMALL[name])
    o.update(10)
    g.update(10)
    for f in FIELDS:
        assert rel(g.get(f), o.get(f)) < 1e-10, (name, f, rel(g.get(f), o.get(f)))
    assert g.status() == 0


def smooth_ic(nav):
    """The reference's smooth initial fields: set_velocity(0.2, 1, 1) and
    set_temperature(0.1, 1, 1) (navier.rs:927-936), zero pressure."""
    nav.set_velocity(0.2, 1.0, 1.0)
    nav.set_temperature(0.1, 1.0, 1.0)
    nav.zero_pressure()


@pytest.mark.parametrize("case", [(O.BOX_ADIABATIC, 64, 64, 1e5, 1.0, 0.02, 1.0),
                                  (O.BOX_CONDUCTING, 48, 40, 1e6, 0.7, 5e-3, 1.5),
                                  (O.PERIODIC, 64, 33, 1e5, 1.0, 5e-3, 1.0)])
def test_smooth_initial_fields(R, case):
    """The initial fields to 1e-13; after 5 steps every field to 1e-10, the
    pseudo pressure to 1e-10 of the pressure's scale: from a smooth start the
    projection's correction potential pres[1] is 3-4 orders of magnitude
    below pres[0] (box 64^2: 3.3e-5 against 0.12), so rounding at the
    pressure's scale is a large part of its own norm."""
    o = O.Navier2D(*case[1:], case[0])
    g = R.Navier2D(*case[1:], case[0], seed=None)
    for x in (o, g):
        smooth_ic(x)
    for f in FIELDS:
        assert rel(g.get(f), o.get(f)) < 1e-13, (f, rel(g.get(f), o.get(f)))
    o.update(5)
    g.update(5)
    for f in (O.TEMP, O.UX, O.UY, O.PRES0):
        assert rel(g.get(f), o.get(f)) < 1e-10, (f, rel(g.get(f), o.get(f)))
    d = np.linalg.norm(g.get(O.PRES1) - o.get(O.PRES1))
    assert d < 1e-10 * np.linalg.norm(o.get(O.PRES0)), (d, np.linalg.norm(o.get(O.PRES1)))


def test_box513_dense_x_transform(R):
    """FP64 box 513 x 513 from the smooth initial fields, 3 steps.  At this size
    the results move with rounding alone by more than 1e-10: a Chebyshev
    derivative amplifies rounding by about n^2 (eps n^2 = 6e-11 at n = 513),
    and the pressures move between two LAPACK-grade decompositions of the
    511-mode Poisson operator.  Both spreads are measured on the oracle (DCT-I
    through the FFT against its defining sum; geev against QZ).  Every field
    must be within 4x the larger spread, and within 1e-10 where both are
    smaller."""
    case = (O.BOX_ADIABATIC, 513, 513, 1e6, 1.0, 1e-3, 1.0)

    def oracle_case():
        o = O.Navier2D(*case[1:], case[0])
        smooth_ic(o)
        return o

    o = oracle_case()
    o.update(3)
    O.set_dense_dct(513)
    try:
        o_dct = oracle_case()
        o_dct.update(3)
    finally:
        O.set_dense_dct(-1)
    from test_gpu_parity import _qz_eig
    orig = O.tensor_eig
    O.tensor_eig = _qz_eig
    try:
        o_qz = oracle_case()
    finally:
        O.tensor_eig = orig
    o_qz.update(3)
    g = R.Navier2D(*case[1:], case[0], seed=None)
    smooth_ic(g)
    g.update(3)
    for f in FIELDS:
        spread = max(rel(o_dct.get(f), o.get(f)), rel(o_qz.get(f), o.get(f)))
        e = rel(g.get(f), o.get(f))
        print("box513", f, "gpu vs oracle", e, "oracle spread (dct, eig)", rel(o_dct.get(f), o.get(f)),
              rel(o_qz.get(f), o.get(f)))
        assert e < max(1e-10, 4.0 * spread), (f, e, spread)
    assert g.status() == 0


@pytest.mark.parametrize("args, precision", [
    ((2048, 65, 1e5, 1.0, 1e-3, 1.0, O.PERIODIC), "fp64"),        # periodic x pass
    ((1025, 1025, 1e5, 1.0, 1e-3, 1.0, O.BOX_ADIABATIC), "fp64"),  # box x pass, dense form too
    ((4096, 65, 1e5, 1.0, 1e-3, 1.0, O.PERIODIC), "mixed"),       # the set-up passes' lanes
])
def test_oversize_refused_at_creation(R, args, precision):
    prec = R.PREC_FP64 if precision == "fp64" else R.PREC_MIXED
    with pytest.raises(R.RbcError) as e:
        R.Navier2D(*args, precision=prec, seed=None)
    assert e.value.code == R.RBC_ERR_INVALID and "shared memory" in str(e.value), str(e.value)
    with pytest.raises(R.RbcError) as e:
        R.Batch([args], precision=prec)
    assert e.value.code == R.RBC_ERR_INVALID


def test_oversize_space_refused(R):
    with pytest.raises(R.RbcError) as e:
        R.Space2(R.Base(O.FOURIER, 8192), R.Base(O.CD, 17))
    assert e.value.code == R.RBC_ERR_INVALID and "shared memory" in str(e.value), str(e.value)


def test_mixed_periodic_beyond_the_fp64_limit(R):
    """Periodic 2048 x 33: the FP64 x pass does not fit a block, the mixed
    form's FP32 x pass does. Three steps against the oracle, at the mixed
    form's precision."""
    o, g = pair(R, O.PERIODIC, 2048, 33, 1e5, 1.0, 5e-3, 4.0, precision=R.PREC_MIXED)
    o.update(3)
    g.update(3)
    for f in (O.TEMP, O.UX, O.UY, O.PRES0):
        assert rel(g.get(f), o.get(f)) < 1e-5, (f, rel(g.get(f), o.get(f)))
    assert g.status() == 0
