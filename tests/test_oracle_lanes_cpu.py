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


# every stage the FFT builds: radix 4, 2, 3, odd primes up to 64 (paired
# butterflies), Bluestein (prime factors above 64), and the odd-length and
# packed even-length real transforms
FFT_LENGTHS = list(range(1, 70)) + [96, 105, 126, 127, 128, 134, 255, 256, 257, 289, 510, 512, 513, 1021, 1024, 2046]


def test_r2c_c2r_all_stage_kinds_match_numpy():
    rng = np.random.default_rng(5)
    for n in FFT_LENGTHS:
        v = rng.standard_normal(n)
        out = np.zeros(n // 2 + 1, dtype=np.complex128)
        O.lib().or_base_forward(O.FOURIER, n, _dp(v), out.ctypes.data_as(DP))
        ref = np.fft.rfft(v)
        assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref)), n
        back = O.base_backward(O.FOURIER, n, ref)
        assert np.max(np.abs(back - np.fft.irfft(ref, n))) <= 1e-13 * np.max(np.abs(v)), n


def test_dct1_fft_equals_defining_sum():
    rng = np.random.default_rng(6)
    for n in [2, 3, 4, 5, 9, 17, 33, 64, 65, 128, 129, 130, 256, 257, 512, 513]:
        x = rng.standard_normal(n)
        a = O.base_forward(O.CHEB, n, x)
        O.set_dense_dct(n)
        try:
            b = O.base_forward(O.CHEB, n, x)
        finally:
            O.set_dense_dct(-1)
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b)), n
