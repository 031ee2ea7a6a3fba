"""Snapshot format (rustpde_gb300.snapshot): round trip of the numpy writer and
reader, and rejection of foreign or truncated files."""
import numpy as np
import pytest

from rustpde_gb300.snapshot import read_snapshot, write_snapshot


def test_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    ds = {"temp/v": rng.standard_normal((8, 9)), "temp/vhat_re": rng.standard_normal((5, 7)),
          "temp/vhat_im": rng.standard_normal((5, 7)), "x": np.linspace(0, 1, 8)}
    p = tmp_path / "s.snap"
    params = {"nx": 8, "ny": 9, "kind": 2, "precision": 1, "dt": 1e-3, "aspect": 1.5}
    scalars = {"time": 0.25, "ra": 1e5, "pr": 0.7, "nu": 0.1, "kappa": 0.2}
    write_snapshot(p, params, scalars, ds)
    s = read_snapshot(p)
    assert s["params"]["nx"] == 8 and s["params"]["kind"] == 2 and s["params"]["aspect"] == 1.5
    assert s["scalars"] == scalars
    for k, v in ds.items():
        assert np.array_equal(s["datasets"][k], v)


def test_rejects_foreign_and_truncated(tmp_path):
    p = tmp_path / "bad.snap"
    p.write_bytes(b"not a snapshot at all" * 10)
    with pytest.raises(ValueError):
        read_snapshot(p)
    q = tmp_path / "t.snap"
    write_snapshot(q, {"nx": 4, "ny": 4, "kind": 0, "dt": 0.1, "aspect": 1.0},
                   {"time": 0, "ra": 1, "pr": 1, "nu": 1, "kappa": 1}, {"a": np.ones((4, 4))})
    q.write_bytes(q.read_bytes()[:-8])
    with pytest.raises(ValueError):
        read_snapshot(q)
