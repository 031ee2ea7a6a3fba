"""integrate() (src/lib.rs:155-187) for Navier2D through rbc_integrate, against
the oracle's restatement of the same loop (oracle.integrate):

* the callback fires at the same simulated times -- bit-identical, since both
  sides add dt in FP64 every step -- and sees Nu within 1e-9 of the oracle;
* the loop stops at max_time after the same number of steps, also where
  max_time is a multiple of dt and eps_dt = dt * 1e-4 decides;
* a NaN put into the temperature through rbc_set_state stops the loop through
  exit() -- the divergence norm is NaN (navier.rs:855-862) -- after the same
  step as the oracle, with status bit 0 set;
* a callback that returns True stops the loop at once.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "box33": (O.BOX_ADIABATIC, 33, 33, 1e5, 1.0, 0.01, 1.0),
    "periodic64x33": (O.PERIODIC, 64, 33, 1e5, 1.0, 0.005, 1.0),
}


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def pair(R, kind, nx, ny, ra, pr, dt, asp, seed=2):
    o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
    O.standard_ic(o, seed)
    g = R.Navier2D(nx, ny, ra, pr, dt, asp, kind, seed=None)
    R.standard_ic(g, seed)
    return o, g


@pytest.mark.parametrize("name", list(CASES))
def test_callback_times_and_values(R, name):
    o, g = pair(R, *CASES[name])
    dt = CASES[name][5]
    max_time, save = 60 * dt, 10 * dt
    rec_o, rec_g = [], []
    n_o = O.integrate(o, dt, max_time, save, lambda p: rec_o.append((p.time, p.eval(O.NU))))
    n_g = R.integrate(g, max_time, save, lambda p: rec_g.append((p.get_time(), p.eval(R.NU))))
    assert n_g == n_o == 60
    assert len(rec_g) == len(rec_o) >= 6
    for (tg, nug), (to, nuo) in zip(rec_g, rec_o):
        assert tg == to
        assert abs(nug - nuo) <= 1e-9 * abs(nuo)
    assert g.get_time() == o.time


@pytest.mark.parametrize("steps", [1, 7, 30])
def test_stop_at_max_time(R, steps):
    o, g = pair(R, *CASES["box33"])
    dt = CASES["box33"][5]
    for max_time in (steps * dt, steps * dt + 0.5 * dt, steps * dt - 0.5 * dt):
        n_o = O.integrate(o, dt, o.time + max_time)
        n_g = R.integrate(g, g.get_time() + max_time)
        assert n_g == n_o, (max_time, n_g, n_o)
        assert g.get_time() == o.time


@pytest.mark.parametrize("name", list(CASES))
def test_nan_stops_through_exit(R, name):
    o, g = pair(R, *CASES[name])
    dt = CASES[name][5]
    O.integrate(o, dt, 3 * dt)
    R.integrate(g, 3 * dt)
    for side in (o, g):
        t = side.get(O.TEMP)
        t[3, 4] = np.nan
        side.set(O.TEMP, t)
    n_o = O.integrate(o, dt, 1000.0)
    n_g = R.integrate(g, 1000.0)
    assert n_g == n_o < 10
    assert g.status() & 1
    assert np.isnan(g.eval(R.DIV_NORM)) and np.isnan(o.eval(O.DIVNORM))


def test_callback_return_stops(R):
    _, g = pair(R, *CASES["box33"])
    dt = CASES["box33"][5]
    seen = []

    def cb(p):
        seen.append(p.get_time())
        return len(seen) == 2

    n = R.integrate(g, 100 * dt, 5 * dt, cb)
    assert n == 10 and len(seen) == 2
