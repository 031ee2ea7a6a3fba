"""Failure detection without a GPU fault (the reference stops integrate() on a
NaN divergence, navier.rs:855-862, and panics on bad input).  Every failure
here is made on the host, or by a bounded device wait that is given no time:

* a lane GEMM whose completion waits get a limit of 0 polls reports a time-out
  (status bit 1) instead of hanging: through fs_lanes_status for the 1-D
  lanes, rbc_status for every case of a mixed batch, and RBC_ERR_CUDA from
  rbc_integrate; with the default limit back, the next launches are correct;
* a NaN put into one case of a batch through rbc_set_state trips that case's
  status word (bit 0) and leaves every other case bit-identical to the same
  steps without it, in FP64 and in the mixed form;
* the serving loop fails only a request that diverges (RBC_ERR_NUMERIC),
  cancels requests queued and mid-flight (RBC_ERR_CANCELLED), and the other
  requests' results equal the same requests served alone.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


@pytest.fixture
def no_wait(R):
    """Lane GEMM waits limited to 0 polls for the test's body; default after."""
    R.set_gemm_wait_limit(0)
    try:
        yield
    finally:
        R.set_gemm_wait_limit(-1)


def test_lanes_gemm_timeout_reported_then_recovers(R):
    n, lanes = 256, 512
    mix = R.Lanes(R.Base(R.CHEB_DIRICHLET, n), R.PREC_MIXED)
    f64 = R.Lanes(R.Base(R.CHEB_DIRICHLET, n), R.PREC_FP64)
    rng = np.random.default_rng(3)
    spec = rng.standard_normal((lanes, mix.m)) * np.exp(-np.arange(mix.m) / 20.0)
    ref = f64.apply(R.OP_BACKWARD, spec)
    d_in = R.DeviceArray.from_host(spec)
    d_out = R.DeviceArray((lanes, mix.n))
    assert mix.status() == 0
    R.set_gemm_wait_limit(0)
    try:
        mix.apply_dev(R.OP_BACKWARD, d_in, d_out, lanes)
        st = mix.status()
    finally:
        R.set_gemm_wait_limit(-1)
    assert st & 2, st
    # the status word was cleared by the read; the process keeps working
    mix.apply_dev(R.OP_BACKWARD, d_in, d_out, lanes)
    assert mix.status() == 0
    out = d_out.to_host()
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) <= 5e-6


def test_mixed_batch_timeout_sets_status_bit(R, no_wait):
    params = [(32, 17, 1e5, 1.0, 5e-3, 1.0, R.PERIODIC), (16, 16, 1e5, 1.0, 1e-2, 1.0, R.BOX_ADIABATIC)]
    b = R.Batch(params, precision=R.PREC_MIXED)
    for i, c in enumerate(b.cases):
        R.standard_ic(c, seed=3 + i)
    b.update(1)
    b.synchronize()
    assert all(c.status() & 2 for c in b.cases), [c.status() for c in b.cases]


def test_integrate_stops_on_gemm_timeout(R):
    c = R.Navier2D(32, 17, 1e5, 1.0, 5e-3, 1.0, R.PERIODIC, precision=R.PREC_MIXED, seed=None)
    R.standard_ic(c, seed=4)
    R.set_gemm_wait_limit(0)
    try:
        with pytest.raises(R.RbcError) as e:
            R.integrate(c, 50 * 5e-3)
    finally:
        R.set_gemm_wait_limit(-1)
    assert e.value.code == R.RBC_ERR_CUDA
    assert c.status() & 2
    # a new case afterwards steps normally (Nu/KE within the mixed tolerance of FP64)
    m = R.Navier2D(32, 17, 1e5, 1.0, 5e-3, 1.0, R.PERIODIC, precision=R.PREC_MIXED, seed=None)
    d = R.Navier2D(32, 17, 1e5, 1.0, 5e-3, 1.0, R.PERIODIC, precision=R.PREC_FP64, seed=None)
    for x in (m, d):
        R.standard_ic(x, seed=4)
        assert R.integrate(x, 20 * 5e-3) == 20
    assert m.status() == 0
    for what in (R.NU, R.KE):
        assert abs(m.eval(what) - d.eval(what)) <= 1e-6 * abs(d.eval(what))


BATCH = [(32, 17, 1e5, 1.0, 5e-3, 1.0, 2), (16, 16, 1e5, 1.0, 1e-2, 1.0, 0),
         (64, 33, 1e6, 0.7, 2e-3, 1.5, 2), (24, 20, 1e5, 7.0, 1e-2, 1.2, 0)]
FIELDS = ("TEMP", "UX", "UY", "PRES", "PSEUDO_PRES")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_one_batch_case_leaves_others_bit_identical(R, precision):
    prec = R.PREC_FP64 if precision == "fp64" else R.PREC_MIXED
    b = R.Batch(BATCH, precision=prec)
    for i, c in enumerate(b.cases):
        R.standard_ic(c, seed=20 + i)
    b.update(2)
    b.synchronize()
    start = R.PinnedArray((b.state_bytes(),), np.uint8)
    b.get_state_all(start.array)
    # the same five steps twice from the same state: clean, then with a NaN in case 1
    b.update(5)
    b.synchronize()
    clean = [{f: c.get(getattr(R, f)) for f in FIELDS} for c in b.cases]
    assert all(c.status() == 0 for c in b.cases)
    b.set_state_all(start.array)
    t = b.cases[1].get(R.TEMP)
    t[3, 4] = np.nan
    b.cases[1].set(R.TEMP, t)
    b.update(5)
    b.synchronize()
    assert b.cases[1].status() & 1
    for i, c in enumerate(b.cases):
        if i == 1:
            continue
        assert c.status() == 0, (i, c.status())
        for f in FIELDS:
            assert np.array_equal(c.get(getattr(R, f)), clean[i][f]), (i, f)


def _serve(R, reqs, cancel_after_start=None, cancel_at_submit=()):
    srv = R.Server(hbm_budget_bytes=8 * 10**9, max_active=8, chunk_steps=4)
    ids = [srv.submit(p, h, seed) for p, h, seed in reqs]
    cancelled = {}
    for k in cancel_at_submit:
        cancelled[ids[k]] = srv.cancel(ids[k])
    if cancel_after_start is not None:
        t0 = time.time()
        while srv.stats()["active"] == 0 and time.time() - t0 < 60:
            time.sleep(0.005)
        time.sleep(0.05)
        cancelled[ids[cancel_after_start]] = srv.cancel(ids[cancel_after_start])
    assert srv.wait_idle(120.0)
    res = {r["id"]: r for r in srv.poll()}
    srv.close()
    return [res[i] for i in ids], cancelled


def test_server_fails_diverging_request_and_cancels(R):
    long_req = ((64, 64, 1e5, 1.0, 0.02, 1.0, 0), 2000.0, 31)          # 100000 steps
    ok = [((64, 33, 1e5, 1.0, 0.005, 1.0, 2), 0.06, 32),
          ((48, 40, 1e5, 7.0, 0.01, 1.2, 0, 1), 0.2, 33)]               # mixed precision
    bad = ((64, 64, 1e8, 1.0, 0.5, 1.0, 2), 20.0, 34)                  # explicit convection blows up
    queued = ((64, 64, 1e5, 1.0, 0.02, 1.0, 2), 1.0, 35)
    reqs = [long_req, ok[0], bad, ok[1], queued]
    res, cancelled = _serve(R, reqs, cancel_after_start=0, cancel_at_submit=(4,))
    assert cancelled == {res[0]["id"]: True, res[4]["id"]: True}
    assert res[0]["status"] == R.RBC_ERR_CANCELLED and 0 < res[0]["steps"] < 100000
    assert res[4]["status"] == R.RBC_ERR_CANCELLED
    assert res[2]["status"] == R.RBC_ERR_NUMERIC
    for k in (1, 3):
        assert res[k]["status"] == 0
        alone, _ = _serve(R, [reqs[k]])
        for key in ("nu", "ke", "steps", "sim_time"):
            assert alone[0][key] == res[k][key], (k, key)
