"""Device selection through the C ABI (rbc_set_device / rbc_get_device): the
library links its own CUDA runtime, so a rank selects its GPU there.  On one
GPU: ordinal 0 is accepted and reported back, an ordinal past the last device
is refused with RBC_ERR_INVALID, and cases created afterwards step normally."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def test_set_and_get_device(R):
    R.set_device(0)
    assert R.get_device() == 0
    with pytest.raises(R.RbcError) as e:
        R.set_device(4096)
    assert e.value.code == R.RBC_ERR_INVALID
    assert R.get_device() == 0
    c = R.Navier2D(16, 16, 1e5, 1.0, 1e-2, 1.0, R.BOX_ADIABATIC, seed=None)
    R.standard_ic(c, seed=1)
    c.update(3)
    assert c.status() == 0
