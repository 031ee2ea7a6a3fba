"""The oracle's batched 1-D lanes and its FFT (test infrastructure checks):

* or_lanes_apply (one basis and one solver for many lanes, the CPU
  counterpart of fs_lanes_apply) gives, lane by lane, exactly what the
  oracle's single-lane functions give;
* the oracle's FFT, with Bluestein's algorithm for lengths that have a prime
  factor above 64, matches numpy's FFT for such lengths and for the direct
  prime stages below that.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

DP = ctypes.POINTER(ctypes.c_double)


def _dp(a):
    return a.ctypes.data_as(DP)


@pytest.mark.parametrize("kind,n", [(O.CD, 24), (O.CN, 33), (O.CHEB, 20), (O.CD, 128)])
def test_lanes_match_single_lane_functions(kind, n):
    L = O.lib()
    m = n - 2 if kind in (O.CD, O.CN) else n
    rng = np.random.default_rng(n + kind)
    spec = rng.standard_normal((3, m))
    phys = rng.standard_normal((3, n))
    single = {0: L.or_base_forward, 1: L.or_base_backward, 2: L.or_base_to_ortho, 3: L.or_base_from_ortho}
    for op, x, ol in ((0, phys, m), (1, spec, n), (2, spec, n), (3, phys, m)):
        got = O.lanes_apply(kind, n, op, x)
        for lane in range(3):
            ref = np.zeros(ol)
            xl = np.ascontiguousarray(x[lane])
            single[op](kind, n, _dp(xl), _dp(ref))
            assert np.array_equal(got[lane], ref), (op, lane)
    if kind in (O.CD, O.CN):
        got = O.lanes_apply(kind, n, 4, phys, c=5e-4)
        for lane in range(3):
            ref = np.zeros(m)
            xl = np.ascontiguousarray(phys[lane])
            L.or_solver1d(kind, n, O.HHOLTZ_ADI, 5e-4, _dp(xl), _dp(ref))
            assert np.array_equal(got[lane], ref)


@pytest.mark.parametrize("n", [22, 94, 194, 202, 254, 510, 1022])
def test_fft_prime_factor_lengths_match_numpy(n):
    v = np.random.default_rng(n).standard_normal(n)
    out = np.zeros(n // 2 + 1, dtype=np.complex128)
    O.lib().or_base_forward(O.FOURIER, n, _dp(v), out.ctypes.data_as(DP))
    ref = np.fft.rfft(v)
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))
