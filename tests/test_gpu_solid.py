"""Solid-mask penalisation on the GPU (navier.rs:551-560, 579-584, 603-608)
against the CPU FP64 oracle on the same seeded inputs and masks.

Tolerance: relative L2 per field <= 1e-10 after 10 steps, as for the plain
step; the mask arithmetic itself is compared at 1e-12 relative.
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


CASES = {
    # name: (kind, nx, ny, ra, pr, dt, aspect, mask)
    "box32_cylinder": (O.BOX_ADIABATIC, 32, 32, 1e5, 1.0, 0.01, 1.0, ("cyl", 0.2, 0.0, 0.2)),
    "box33_cond_rough": (O.BOX_CONDUCTING, 33, 33, 1e5, 1.0, 0.005, 1.5, ("rough", 0.1, 6.0)),
    "box65_porosity": (O.BOX_ADIABATIC, 65, 65, 1e6, 0.7, 0.002, 1.0, ("poro", 0.3, 0.6)),
    "periodic64x33_cylinder": (O.PERIODIC, 64, 33, 1e5, 1.0, 0.005, 1.0, ("cyl", 3.0, 0.0, 0.3)),
    "periodic128x65_rough": (O.PERIODIC, 128, 65, 1e6, 1.0, 0.002, 2.0, ("rough", 0.1, 2.0)),
}


def make_mask(spec, x, y):
    if spec[0] == "cyl":
        return O.solid_cylinder_inner(x, y, *spec[1:])
    if spec[0] == "rough":
        return O.solid_roughness_sinusoid(x, y, *spec[1:])
    return O.solid_porosity(x, y, *spec[1:])


def pair(R, name, seed=4):
    kind, nx, ny, ra, pr, dt, asp, spec = CASES[name]
    o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
    O.standard_ic(o, seed)
    g = R.Navier2D(nx, ny, ra, pr, dt, asp, kind, seed=None)
    R.standard_ic(g, seed)
    x, y = o.coords(O.TEMP)
    m, v = make_mask(spec, x, y)
    o.set_solid(m, v)
    g.solid = [m, v]
    return o, g


@pytest.mark.parametrize("name", list(CASES))
def test_ten_steps_with_solid(R, name):
    o, g = pair(R, name)
    o.update(10)
    g.update(10)
    for f in FIELDS:
        e = rel(g.get(f), o.get(f))
        assert e < 1e-10, (name, f, e)
    assert g.status() == 0


def test_solid_round_trip_and_removal(R):
    o, g = pair(R, "box32_cylinder")
    m, v = g.solid
    x, y = o.coords(O.TEMP)
    mo, vo = O.solid_cylinder_inner(x, y, 0.2, 0.0, 0.2)
    np.testing.assert_array_equal(m, mo)
    np.testing.assert_array_equal(v, vo)
    # removing the solid restores the plain step
    g.solid = None
    o.set_solid(None)
    assert g.solid is None
    o.update(5)
    g.update(5)
    for f in FIELDS:
        assert rel(g.get(f), o.get(f)) < 1e-10


def test_solid_changes_the_flow(R):
    """The damping term is active: with and without the mask differ."""
    _, g = pair(R, "box32_cylinder")
    h = R.Navier2D(32, 32, 1e5, 1.0, 0.01, 1.0, O.BOX_ADIABATIC, seed=None)
    R.standard_ic(h, 4)
    g.update(5)
    h.update(5)
    assert rel(g.get(O.UX), h.get(O.UX)) > 1e-3


def test_solid_unsupported_forms(R):
    # the mixed form has no solid lane, in a batch or alone (FP64 batches take masks)
    params = [(32, 17, 1e5, 1.0, 0.005, 1.0, R.PERIODIC)] * 2
    b = R.Batch(params, precision=R.PREC_MIXED)
    m = np.zeros((32, 17))
    with pytest.raises(R.RbcError) as e:
        b.cases[0].solid = [m, m]
    assert e.value.code == R.RBC_ERR_UNSUPPORTED
    g = R.Navier2D(32, 17, 1e5, 1.0, 0.005, 1.0, R.PERIODIC, precision=R.PREC_MIXED, seed=None)
    with pytest.raises(R.RbcError) as e:
        g.solid = [m, m]
    assert e.value.code == R.RBC_ERR_UNSUPPORTED
    h = R.Navier2D(32, 17, 1e5, 1.0, 0.005, 1.0, R.PERIODIC, seed=None)
    with pytest.raises(ValueError):
        h.solid = [np.zeros((31, 17)), np.zeros((31, 17))]


@pytest.mark.parametrize("nx,ny", [(33, 33), (64, 48), (129, 65)])
def test_porosity_interpolate(R, nx, ny):
    from rustpde_gb300 import solid_masks as S
    a = S.solid_porosity_interpolate(nx, ny, 0.2, 0.7)
    b = O.solid_porosity_interpolate(nx, ny, 0.2, 0.7)
    for p, q in zip(a, b):
        assert np.abs(p - q).max() <= 1e-12 * max(np.abs(q).max(), 1.0)


def test_snapshot_carries_the_mask(R, tmp_path):
    """Navier2D::write stores the mask as dataset solid/mask (navier.rs:998-1001)."""
    from rustpde_gb300.snapshot import read_snapshot
    o, g = pair(R, "periodic64x33_cylinder")
    path = str(tmp_path / "flow.rbc")
    g.write(path)
    snap = read_snapshot(path)
    np.testing.assert_array_equal(snap["datasets"]["solid/mask"], g.solid[0])


def test_solid_in_fp64_batch_equals_alone(R):
    """A solid mask set on a case of an FP64 batch: the batch rebuilds that
    group's plan and its graphs, and every case steps bitwise as it does alone
    (with and without its mask); removing the mask restores the plain step."""
    names = ["box32_cylinder", "periodic64x33_cylinder"]
    params = [CASES[n][1:7] + (CASES[n][0],) for n in names] + [(16, 16, 1e5, 1.0, 1e-2, 1.0, O.BOX_ADIABATIC)]
    b = R.Batch(params)
    singles = [R.Navier2D(*p, seed=None) for p in params]
    masks = []
    for k, n in enumerate(names):
        o = O.Navier2D(*params[k])
        x, y = o.coords(O.TEMP)
        masks.append(make_mask(CASES[n][7], x, y))
    for i in range(len(params)):
        R.standard_ic(b.cases[i], seed=30 + i)
        R.standard_ic(singles[i], seed=30 + i)
    for k in range(len(names)):
        b.cases[k].solid = list(masks[k])
        singles[k].solid = list(masks[k])
    b.update(4)
    for s in singles:
        s.update(4)
    b.synchronize()
    for i, s in enumerate(singles):
        for f in FIELDS:
            assert np.array_equal(b.cases[i].get(f), s.get(f)), (i, f)
    # without the mask again: the plain step on both sides
    b.cases[0].solid = None
    singles[0].solid = None
    b.update(2)
    singles[0].update(2)
    b.synchronize()
    for f in FIELDS:
        assert np.array_equal(b.cases[0].get(f), singles[0].get(f)), f


def test_mask_toggles_hold_device_memory(R):
    """Setting and removing a mask re-plans the x pass; the step tables of the
    old plan are freed, so device memory stays level over many changes, and
    the step after them still follows the oracle."""
    o, g = pair(R, "periodic64x33_cylinder")
    m, v = g.solid
    held = g.device_bytes()
    for _ in range(25):
        g.solid = None
        g.solid = [m, v]
        assert g.device_bytes() == held
    o.update(4)
    g.update(4)
    for f in FIELDS:
        assert rel(g.get(f), o.get(f)) < 1e-10, f


def test_mask_toggles_in_fp64_batch(R):
    """The batch's re-planned groups free their old tables too; after many
    changes its case still steps bitwise as the case alone."""
    p = CASES["box32_cylinder"]
    params = [p[1:7] + (p[0],), (16, 16, 1e5, 1.0, 1e-2, 1.0, O.BOX_ADIABATIC)]
    b = R.Batch(params)
    s = R.Navier2D(*params[0], seed=None)
    R.standard_ic(b.cases[0], seed=7)
    R.standard_ic(s, seed=7)
    o = O.Navier2D(*params[0])
    x, y = o.coords(O.TEMP)
    m, v = make_mask(p[7], x, y)
    for _ in range(10):
        b.cases[0].solid = [m, v]
        b.cases[0].solid = None
    b.cases[0].solid = [m, v]
    s.solid = [m, v]
    b.update(3)
    s.update(3)
    b.synchronize()
    for f in FIELDS:
        assert np.array_equal(b.cases[0].get(f), s.get(f)), f
