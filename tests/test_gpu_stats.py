"""Statistics (src/navier/statistics.rs) and the diagnostics series of
Navier2D::callback (navier.rs:819-838) on the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P = (64, 33, 1e5, 1.0, 5e-3, 1.0, 2)
B = (48, 40, 1e5, 0.7, 1e-2, 1.5, 0)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def _case(R, params, steps):
    c = R.Navier2D(*params, seed=None)
    R.standard_ic(c, 5)
    c.update(steps)
    return c


@pytest.mark.parametrize("params", [P, B])
def test_running_mean_and_counters(R, params):
    a = _case(R, params, 2)
    a.stats_reset()
    a.stats_update()          # that(t2)
    a.update(3)
    a.stats_update()          # that(t5)
    t2 = _case(R, params, 2)
    t2.stats_reset()
    t2.stats_update()
    t5 = _case(R, params, 5)
    t5.stats_reset()
    t5.stats_update()
    m = a.stats_get(0)
    ref = (t2.stats_get(0) * 1.0 + t5.stats_get(0)) / 2.0
    assert np.allclose(m, ref, rtol=0, atol=1e-14 * np.abs(ref).max())
    # ux, uy and the Nusselt field are the latest, not averaged (statistics.rs:145-147)
    for k in (1, 2, 3):
        assert np.array_equal(a.stats_get(k), t5.stats_get(k))
    info = a.stats_info()
    assert info["num_save"] == 2
    assert abs(info["tot_time"] - a.get_time()) < 1e-15
    assert abs(info["avg_time"] - 3 * params[4]) < 1e-12


@pytest.mark.parametrize("params", [P, B])
def test_nusselt_field_averages_to_nuvol(R, params, tmp_path):
    from rustpde_gb300.snapshot import read_snapshot
    c = _case(R, params, 4)
    c.stats_reset()
    c.stats_update()
    p = str(tmp_path / "stats.snap")
    c.stats_write(p)
    s = read_snapshot(p)["datasets"]
    x, dx, y, dy = s["x"], s["dx"], s["y"], s["dy"]
    wx = dx / abs(x[-1] - x[0])  # average.rs weights (dx / length), as rbc_eval uses
    wy = dy / abs(y[-1] - y[0])
    v = s["nusselt/v"]
    avg = float(wx @ v @ wy)
    nuvol = c.eval(R.NUVOL)
    assert abs(avg - nuvol) <= 1e-10 * abs(nuvol), (avg, nuvol)
    assert s["num_save"][0] == 1.0


def test_diagnostics_series(R):
    c = _case(R, P, 1)
    want = []
    for _ in range(3):
        c.diag_record()
        want.append((c.get_time(), c.eval(R.NU), c.eval(R.NUVOL), c.eval(R.RE)))
        c.update(2)
    d = c.diag_series()
    assert len(d["time"]) == 3
    for k, (t, nu, nuv, re) in enumerate(want):
        assert d["time"][k] == t and d["nu"][k] == nu and d["nuvol"][k] == nuv and d["re"][k] == re
