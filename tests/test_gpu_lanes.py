"""Batched 1-D transforms and Helmholtz solves (fs_lanes_*).

* FP64 form against the oracle, lane by lane (1e-12).
* Mixed form (tensor-core 3xTF32 dense products, FP64 banded sweep) against
  the FP64 form on the precision-microbenchmark workload: 4096 lanes of length
  N in {128, 256, 512}, spectral coefficients g_k exp(-k/20) with g ~ N(0, 1).
  The relative L2 error of every stage must stay below MIXED_TOL.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 5e-6    # relative L2 per stage, 3xTF32 with FP32 accumulation (grows like sqrt(N))
FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    oracle.build()
    return oracle


def _spectral(rng, lanes, m):
    k = np.arange(m)
    return rng.standard_normal((lanes, m)) * np.exp(-k / 20.0)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("kind,n", [(0, 33), (1, 33), (2, 64), (1, 130), (0, 48)])
def test_fp64_lanes_match_oracle(R, O, kind, n):
    rng = np.random.default_rng(n + 10 * kind)
    L = R.Lanes(R.Base(kind, n), R.PREC_FP64, hholtz_c=5e-4 if kind else None)
    lanes = 6
    spec = _spectral(rng, lanes, L.m)
    phys = rng.standard_normal((lanes, n))
    cases = [
        (R.OP_FORWARD, phys, lambda v: O.base_forward(kind, n, v)),
        (R.OP_BACKWARD, spec, lambda v: O.base_backward(kind, n, v)),
        (R.OP_TO_ORTHO, spec, lambda v: O.base_to_ortho(kind, n, v)),
        (R.OP_FROM_ORTHO, phys, lambda v: O.base_from_ortho(kind, n, v)),
    ]
    if kind:
        cases.append((R.OP_HHOLTZ, phys, lambda v: O.solver1d(kind, n, O.HHOLTZ_ADI, 5e-4, v)))
    for op, x, ref in cases:
        got = L.apply(op, x)
        want = np.stack([ref(x[i]) for i in range(lanes)])
        assert got.shape == want.shape
        err = np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300)
        assert err <= FP64_TOL, (op, err)


@pytest.mark.parametrize("n", [128, 256, 512])
@pytest.mark.parametrize("kind", [0, 1])
def test_mixed_lanes_vs_fp64(R, kind, n):
    rng = np.random.default_rng(1000 + n + kind)
    c = 5e-4  # dt/2 with dt = 1e-3
    f64 = R.Lanes(R.Base(kind, n), R.PREC_FP64, hholtz_c=c if kind else None)
    mix = R.Lanes(R.Base(kind, n), R.PREC_MIXED, hholtz_c=c if kind else None)
    lanes = 4096
    spec = _spectral(rng, lanes, f64.m)
    phys = f64.apply(R.OP_BACKWARD, spec)
    ortho = f64.apply(R.OP_TO_ORTHO, spec)
    ops = [(R.OP_FORWARD, phys), (R.OP_BACKWARD, spec), (R.OP_TO_ORTHO, spec), (R.OP_FROM_ORTHO, ortho)]
    if kind:
        ops.append((R.OP_HHOLTZ, ortho))
    errs = {}
    for op, x in ops:
        errs[op] = _rel(mix.apply(op, x), f64.apply(op, x))
    print(f"kind {kind} n {n} relative L2 errors per op: {errs}")
    for op, e in errs.items():
        assert e <= MIXED_TOL, (op, e)


def test_mixed_lanes_partial_tile(R):
    # lane counts that are not multiples of the 128-lane tile, odd lengths
    rng = np.random.default_rng(5)
    f64 = R.Lanes(R.Base(1, 70), R.PREC_FP64)
    mix = R.Lanes(R.Base(1, 70), R.PREC_MIXED)
    for lanes in (1, 127, 129, 300):
        spec = _spectral(rng, lanes, f64.m)
        a = mix.apply(R.OP_BACKWARD, spec)
        b = f64.apply(R.OP_BACKWARD, spec)
        assert _rel(a, b) <= MIXED_TOL
