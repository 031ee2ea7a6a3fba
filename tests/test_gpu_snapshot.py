"""Snapshots (Navier2D::write / read, navier.rs:961-1013): the written datasets
equal the case's state and physical fields; reading restores a case exactly
(a restarted run continues bit for bit); a snapshot of another resolution is
broadcast (low modes copied, the rest zero, field/read.rs:116-125)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def _case(R, params, steps, seed=3):
    c = R.Navier2D(*params, seed=None)
    R.standard_ic(c, seed)
    c.update(steps)
    return c


@pytest.mark.parametrize("params", [(64, 33, 1e5, 1.0, 5e-3, 1.0, 2), (48, 40, 1e5, 0.7, 1e-2, 1.5, 0)])
def test_write_matches_state_and_read_restores(R, tmp_path, params):
    from rustpde_gb300.snapshot import read_snapshot
    c = _case(R, params, 5)
    p = str(tmp_path / "a.snap")
    c.write(p)
    s = read_snapshot(p)
    assert abs(s["scalars"]["time"] - c.get_time()) == 0.0
    cplx = params[6] == 2
    for name, fid in (("temp", R.TEMP), ("ux", R.UX), ("uy", R.UY), ("pres", R.PRES)):
        vh = c.get(fid)
        if cplx:
            assert np.array_equal(s["datasets"][name + "/vhat_re"], vh.real)
            assert np.array_equal(s["datasets"][name + "/vhat_im"], vh.imag)
        else:
            assert np.array_equal(s["datasets"][name + "/vhat"], vh)
        v = c.get_physical(fid)
        if fid == R.TEMP:
            v = v + c.get_physical(R.FIELDBC)
        assert np.allclose(s["datasets"][name + "/v"], v, rtol=0, atol=1e-13)
    # restart: a fresh case reads the snapshot and continues identically
    d = R.Navier2D(*params, seed=None)
    d.read(p)
    assert d.get_time() == c.get_time()
    for fid in (R.TEMP, R.UX, R.UY, R.PRES):
        assert np.array_equal(d.get(fid), c.get(fid))
    # pres[1] is not part of a snapshot (the reference writes pres[0] only);
    # copy it so that the continued runs start from the same state
    d.set(R.PSEUDO_PRES, c.get(R.PSEUDO_PRES))
    c.update(3)
    d.update(3)
    for fid in (R.TEMP, R.UX, R.UY, R.PRES, R.PSEUDO_PRES):
        assert np.array_equal(d.get(fid), c.get(fid))


def test_read_broadcasts_resolution(R, tmp_path):
    small = (64, 33, 1e5, 1.0, 5e-3, 1.0, 2)
    big = (128, 65, 1e5, 1.0, 5e-3, 1.0, 2)
    c = _case(R, small, 2)
    p = str(tmp_path / "b.snap")
    c.write(p)
    d = R.Navier2D(*big, seed=None)
    d.read(p)
    for fid in (R.TEMP, R.UX, R.UY, R.PRES):
        a, b = c.get(fid), d.get(fid)
        r, q = a.shape
        assert np.array_equal(b[:r, :q], a)
        assert not np.any(b[r:, :]) and not np.any(b[:, q:])


def test_python_written_snapshot_is_read(R, tmp_path):
    from rustpde_gb300.snapshot import read_snapshot, write_snapshot
    params = (48, 40, 1e5, 0.7, 1e-2, 1.5, 0)
    c = _case(R, params, 2)
    p = str(tmp_path / "c.snap")
    c.write(p)
    s = read_snapshot(p)
    s["datasets"]["temp/vhat"] = s["datasets"]["temp/vhat"] * 2.0
    s["scalars"]["time"] = 7.5
    q = str(tmp_path / "d.snap")
    write_snapshot(q, s["params"], s["scalars"], s["datasets"])
    d = R.Navier2D(*params, seed=None)
    d.read(q)
    assert d.get_time() == 7.5
    assert np.array_equal(d.get(R.TEMP), 2.0 * c.get(R.TEMP))
