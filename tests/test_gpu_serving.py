"""Serving loop (rbc_server_*): continuous batching of RBC solve requests.

* every request's result (Nu and KE at its horizon) is the same when it is
  served alone and when it shares the device with other requests that arrive
  while it runs (tolerance 0: no kernel combines data of two cases);
* the results equal the same case stepped on its own through rbc_step;
* requests that can never fit the memory budget fail with RBC_ERR_NOMEM
  without stopping the loop.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 0.0


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


REQS = [  # (params, horizon, seed)
    ((64, 64, 1e5, 1.0, 0.02, 1.0, 0), 0.3, 11),
    ((64, 33, 1e5, 1.0, 0.005, 1.0, 2), 0.06, 12),
    ((128, 64, 1e6, 0.7, 2e-3, 1.5, 2), 0.05, 13),
    ((48, 40, 1e6, 7.0, 5e-3, 1.2, 1), 0.11, 14),
    ((64, 64, 1e5, 1.0, 0.02, 1.0, 0, 1), 0.3, 15),      # mixed precision
    ((128, 65, 1e6, 1.0, 4e-3, 2.0, 2, 1), 0.07, 16),     # mixed precision
]


def serve(R, reqs, stagger=0.0):
    srv = R.Server(hbm_budget_bytes=8 * 10**9, max_active=8, chunk_steps=4)
    ids = []
    for p, h, seed in reqs:
        ids.append(srv.submit(p, h, seed))
        if stagger:
            time.sleep(stagger)
    assert srv.wait_idle(120.0)
    res = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    return [res[i] for i in ids], st


def test_alone_equals_in_mix(R):
    mixed, st = serve(R, REQS, stagger=0.01)
    assert st["rebuilds"] >= 2  # the active set changed while cases were running
    for k, req in enumerate(REQS):
        alone, _ = serve(R, [req])
        a, b = alone[0], mixed[k]
        assert a["status"] == 0 and b["status"] == 0
        assert a["steps"] == b["steps"] == max(1, round(req[1] / req[0][4]))
        for key in ("nu", "ke", "sim_time"):
            assert abs(a[key] - b[key]) <= TOL * abs(a[key]), (k, key, a[key], b[key])


def test_served_equals_single_case(R):
    res, _ = serve(R, REQS[:4])
    for (p, h, seed), r in zip(REQS[:4], res):
        c = R.Navier2D(*p[:7], precision=p[7] if len(p) > 7 else R.PREC_FP64, seed=None)
        c.set_velocity(0.2, 1.0, 1.0)
        c.set_temperature_noise(1e-3, seed)
        c.update(r["steps"])
        assert c.eval(R.NU) == r["nu"] and c.eval(R.KE) == r["ke"]


def test_fused_y2_form_served(R, monkeypatch):
    # RBC_SERVER_FORM=3 runs the periodic Y2 pass as one launch, gated per
    # case like the three launches of form 2 (the short request finishes while
    # its group still runs): bitwise the same results
    reqs = [((128, 65, 1e6, 1.0, 4e-3, 2.0, 2, 1), 0.07, 16), ((64, 33, 1e5, 1.0, 5e-3, 1.0, 2, 1), 0.02, 17),
            ((64, 64, 1e5, 1.0, 0.02, 1.0, 0, 1), 0.1, 18)]
    out = {}
    for form in ("2", "3"):
        monkeypatch.setenv("RBC_SERVER_FORM", form)
        out[form], _ = serve(R, reqs)
    for a, b in zip(out["2"], out["3"]):
        assert a["status"] == 0 and b["status"] == 0
        for key in ("nu", "ke", "sim_time"):
            assert a[key] == b[key], (key, a[key], b[key])


def test_budget_rejection(R):
    srv = R.Server(hbm_budget_bytes=1 << 20, max_active=4, chunk_steps=2)
    rid = srv.submit((64, 64, 1e5, 1.0, 0.02, 1.0, 0), 0.1, 1)
    assert srv.wait_idle(60.0)
    out = srv.poll()
    srv.close()
    assert len(out) == 1 and out[0]["id"] == rid and out[0]["status"] == -5


def test_admission_under_memory_pressure(R):
    """A budget of about two cases' worth: every request still completes, the
    device bytes held by the loop (reservations of cases being built, built
    and active cases) never exceed the budget, and each result equals the
    request served alone with a large budget."""
    budget = 24 * 10**6
    reqs = [((64, 64, 1e5, 1.0, 0.02, 1.0, 0), 0.1, 40 + k) for k in range(5)]
    srv = R.Server(hbm_budget_bytes=budget, max_active=8, chunk_steps=4)
    ids = [srv.submit(p, h, seed) for p, h, seed in reqs]
    assert srv.wait_idle(120.0)
    res = {r["id"]: r for r in srv.poll()}
    st = srv.stats()
    srv.close()
    assert 0 < st["peak_bytes_in_use"] <= budget
    for k, rid in enumerate(ids):
        r = res[rid]
        assert r["status"] == 0 and r["steps"] == 5
        alone, _ = serve(R, [reqs[k]])
        assert alone[0]["nu"] == r["nu"] and alone[0]["ke"] == r["ke"]


def test_request_records(R, tmp_path):
    # one JSON line per request: its sizes and parameters, steps, wall time, Nu, KE, status
    import json
    srv = R.Server(hbm_budget_bytes=8 * 10**9, max_active=8, chunk_steps=4)
    ids = [srv.submit(p, h, seed) for p, h, seed in REQS[:3]]
    assert srv.wait_idle(120.0)
    res = srv.poll()
    assert not srv._requests  # delivered requests leave the table: it holds those in flight only
    path = tmp_path / "requests.jsonl"
    srv.write_records(str(path), res)
    srv.close()
    lines = [json.loads(x) for x in path.read_text().splitlines()]
    assert sorted(r["id"] for r in lines) == sorted(ids)
    for rec in lines:
        p, h, seed = REQS[ids.index(rec["id"])]
        assert (rec["nx"], rec["ny"], rec["kind"]) == (p[0], p[1], p[6]) and rec["seed"] == seed
        assert rec["status"] == 0 and rec["steps"] == max(1, round(h / p[4])) and rec["wall_s"] > 0
        assert np.isfinite(rec["nu"]) and np.isfinite(rec["ke"])
