"""Batched form: cases of uneven size and kind advanced together must give
exactly the results of the same cases stepped one by one (the same kernels run
the same lane computations; only the work tables differ), and match the
oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = [
    (64, 64, 1e5, 1.0, 0.02, 1.0, 0),     # config 0
    (32, 17, 1e5, 0.7, 5e-3, 1.5, 2),     # periodic
    (33, 33, 1e6, 7.0, 1e-2, 1.2, 1),     # box conducting
    (64, 64, 1e5, 1.0, 0.02, 1.0, 0),     # same bucket as case 0, other seed
    (64, 33, 1e5, 1.0, 5e-3, 2.0, 2),     # periodic, other size
]
FIELDS = (0, 1, 2, 3, 4)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def test_batch_equals_single_cases(R):
    b = R.Batch(PARAMS)
    nb, nl = b.layout()
    assert nb == 2  # box cases of every size in one group, periodic cases in the other
    singles = []
    for i, p in enumerate(PARAMS):
        R.standard_ic(b.cases[i], seed=10 + i)
        s = R.Navier2D(*p, seed=None)
        R.standard_ic(s, seed=10 + i)
        singles.append(s)
    b.update(6)
    for s in singles:
        s.update(6)
    b.synchronize()
    for i, s in enumerate(singles):
        for f in FIELDS:
            assert np.array_equal(b.cases[i].get(f), s.get(f)), (i, f)
        assert b.cases[i].get_time() == pytest.approx(6 * PARAMS[i][4])


def test_batch_against_oracle(R):
    from oracle import oracle as O
    b = R.Batch(PARAMS[:3])
    for i in range(3):
        R.standard_ic(b.cases[i], seed=3)
    b.update(10)
    for i, p in enumerate(PARAMS[:3]):
        o = O.Navier2D(*p)
        O.standard_ic(o, 3)
        o.update(10)
        for f in FIELDS:
            a, ref = b.cases[i].get(f), o.get(f)
            assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < 1e-10, (i, f)
        assert abs(b.cases[i].eval_nu() - o.eval_nu()) < 1e-10 * abs(o.eval_nu())


def test_batch_case_handles_are_borrowed(R):
    b = R.Batch(PARAMS[:2])
    assert R.lib().rbc_step(b.cases[0]._h, 1) == R.RBC_ERR_INVALID
    assert R.lib().rbc_destroy(b.cases[0]._h) == R.RBC_ERR_INVALID
    assert R.lib().rbc_integrate(b.cases[0]._h, 1.0, 0.0, R.CALLBACK(lambda *a: 0), None, None) == R.RBC_ERR_INVALID


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_io_equals_set_step_get(R, precision):
    # rbc_batch_step_io (each group copied in, stepped and copied back on its
    # own branch) gives bitwise the state of set_state_all + update + get_state_all
    prec = R.PREC_FP64 if precision == "fp64" else R.PREC_MIXED
    bs = [R.Batch(PARAMS, precision=prec) for _ in range(2)]
    for b in bs:
        for i in range(len(PARAMS)):
            R.standard_ic(b.cases[i], seed=30 + i)
        b.update(1)
        b.synchronize()
    n = bs[0].state_bytes()
    # each group's cases hold one contiguous range; every case has its own range
    offs = sorted((bs[0].state_offset(i), i) for i in range(len(PARAMS)))
    assert offs[0][0] == 0 and len({o for o, _ in offs}) == len(PARAMS)
    def group(p):  # kind, and for mixed cases whether every Chebyshev length is 2^p + 1
        pow2 = lambda v: v > 0 and v & (v - 1) == 0
        bfly = precision == "mixed" and pow2(p[1] - 1) and (p[6] == 2 or pow2(p[0] - 1))
        return (p[6] == 2, bfly)
    order = []
    for _, i in offs:
        g = group(PARAMS[i])
        if not order or order[-1] != g:
            assert g not in order, "a group's cases are not contiguous"
            order.append(g)
    start = R.PinnedArray((n,), np.uint8)
    bs[0].get_state_all(start.array)
    ref = R.PinnedArray((n,), np.uint8)
    bs[0].set_state_all(start.array)
    bs[0].update(3)
    bs[0].get_state_all(ref.array)
    out = R.PinnedArray((n,), np.uint8)
    bs[1].step_io(start.array, out.array, 3)
    assert np.array_equal(ref.array, out.array)
    for i in range(len(PARAMS)):
        assert bs[0].cases[i].get_time() == bs[1].cases[i].get_time()
        for f in FIELDS:
            assert np.array_equal(bs[0].cases[i].get(f), bs[1].cases[i].get(f)), (i, f)
    # in place (host_in is host_out), one step
    bs[1].step_io(out.array, out.array, 1)
    bs[0].update(1)
    bs[0].get_state_all(ref.array)
    assert np.array_equal(ref.array, out.array)
