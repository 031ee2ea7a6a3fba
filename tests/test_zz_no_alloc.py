"""fs_forward_noalloc: the forward transform with its intermediate array in the
library's fixed device scratch instead of the space's own.  It must give the
results of fs_forward (same kernels, same inputs: tolerance 0, bit-identical),
on two calls in a row, allocate nothing, and refuse spaces whose intermediate
does not fit the fixed scratch.

Kept in its own file, collected last, so that it runs both alone in a fresh
process (the first call does the per-device set-up) and after the other GPU
tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 0.0  # same kernels on the same inputs: bit-identical

# (base0, n0, base1, n1): Fourier x Dirichlet (periodic velocity space),
# Dirichlet x Neumann (box temperature space), Chebyshev 512 x 257
SPACES = [(5, 64, 1, 33), (1, 64, 2, 64), (0, 512, 0, 257)]


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def _mem_free():
    torch = pytest.importorskip("torch")
    free, _ = torch.cuda.mem_get_info()
    return free


@pytest.mark.parametrize("sp", SPACES)
def test_noalloc_matches_fs_forward_twice(R, sp):
    k0, n0, k1, n1 = sp
    s = R.Space2(R.Base(k0, n0), R.Base(k1, n1))
    rng = np.random.default_rng(7 + n0 + n1)
    for call in range(2):
        v = rng.standard_normal(s.physical)
        d_in = R.DeviceArray.from_host(v)
        d_ref = R.DeviceArray(s.spectral, s.is_complex)
        d_out = R.DeviceArray(s.spectral, s.is_complex)
        s.forward_dev(d_in, d_ref)
        s.forward_noalloc_dev(d_in, d_out)
        R._check(R.lib().rbc_device_synchronize())
        ref, out = d_ref.to_host(), d_out.to_host()
        assert out.shape == ref.shape
        err = np.max(np.abs(out - ref))
        assert err <= TOL * max(1.0, np.max(np.abs(ref))), f"call {call}: max |diff| {err}"


def test_noalloc_allocates_nothing(R):
    """Free device memory is unchanged across three calls.  mem_get_info
    reports the whole device at the allocator's page granularity (2 MiB), so
    this rules out allocations of a page or more, not smaller ones; that the
    entry point calls no allocator at all is a property of its code."""
    s = R.Space2(R.Base(0, 512), R.Base(0, 257))
    v = np.random.default_rng(3).standard_normal(s.physical)
    d_in = R.DeviceArray.from_host(v)
    d_out = R.DeviceArray(s.spectral, s.is_complex)
    s.forward_noalloc_dev(d_in, d_out)  # first call: per-device set-up
    R._check(R.lib().rbc_device_synchronize())
    before = _mem_free()
    for _ in range(3):
        s.forward_noalloc_dev(d_in, d_out)
    R._check(R.lib().rbc_device_synchronize())
    assert _mem_free() == before


def test_noalloc_exact_limit_accepted_one_more_column_refused(R):
    """Chebyshev 512 x 1024: the intermediate is 512 * 1024 doubles, exactly the
    4 MiB of fixed scratch, and is accepted (bit-identical to fs_forward); one
    more column (512 x 1025) is refused before anything is enqueued."""
    s = R.Space2(R.Base(0, 512), R.Base(0, 1024))
    assert s.physical[0] * s.spectral[1] * 8 == 4 * 1024 * 1024
    v = np.random.default_rng(5).standard_normal(s.physical)
    d_in = R.DeviceArray.from_host(v)
    d_ref = R.DeviceArray(s.spectral, s.is_complex)
    d_out = R.DeviceArray(s.spectral, s.is_complex)
    s.forward_dev(d_in, d_ref)
    s.forward_noalloc_dev(d_in, d_out)
    R._check(R.lib().rbc_device_synchronize())
    assert np.array_equal(d_out.to_host(), d_ref.to_host())
    s2 = R.Space2(R.Base(0, 512), R.Base(0, 1025))
    d_in2 = R.DeviceArray(s2.physical, False)
    d_out2 = R.DeviceArray(s2.spectral, s2.is_complex)
    with pytest.raises(R.RbcError) as e:
        s2.forward_noalloc_dev(d_in2, d_out2)
    assert e.value.code == -1


def test_noalloc_rejects_oversized_space(R):
    # 1025 x 1025 doubles of intermediate = 8.4 MB > the 4 MiB fixed scratch
    s = R.Space2(R.Base(0, 1025), R.Base(0, 1025))
    d_in = R.DeviceArray(s.physical, False)
    d_out = R.DeviceArray(s.spectral, s.is_complex)
    with pytest.raises(R.RbcError) as e:
        s.forward_noalloc_dev(d_in, d_out)
    assert e.value.code == -1
    assert "fixed" in str(e.value)
