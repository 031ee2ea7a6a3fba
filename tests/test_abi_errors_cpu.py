"""Error behaviour of the C ABI that needs no GPU: invalid arguments are
refused with RBC_ERR_INVALID and a message (rbc_last_error) before any device
work, and nothing aborts the process.  The reference panics on the same
inputs (funspace/src/utils.rs:63-75, fdma_tensor.rs:173-209)."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


def params(R, **kw):
    p = dict(nx=64, ny=64, ra=1e5, pr=1.0, dt=0.02, aspect=1.0, kind=R.BOX_ADIABATIC, precision=R.PREC_FP64)
    p.update(kw)
    return R.RbcParams(**p)


def last_error(R):
    return R.lib().rbc_last_error().decode()


@pytest.mark.parametrize("kw, word", [
    (dict(kind=7), "kind"),
    (dict(ra=-1.0), "positive"),
    (dict(dt=0.0), "positive"),
    (dict(ny=4), "ny"),
    (dict(nx=6, kind=2), "periodic nx"),
    (dict(nx=4), "nx"),
    (dict(precision=5), "precision"),
])
def test_create_refuses_invalid_params(R, kw, word):
    h = ctypes.c_void_p()
    rc = R.lib().rbc_create(ctypes.byref(params(R, **kw)), ctypes.byref(h))
    assert rc == R.RBC_ERR_INVALID
    assert h.value is None
    assert word in last_error(R)


def test_null_arguments_are_refused(R):
    L = R.lib()
    h = ctypes.c_void_p()
    assert L.rbc_create(None, ctypes.byref(h)) == R.RBC_ERR_INVALID
    assert "null" in last_error(R)
    assert L.rbc_batch_create(None, 3, ctypes.byref(h)) == R.RBC_ERR_INVALID
    buf = ctypes.create_string_buffer(16)
    assert L.rbc_batch_tuning_forms(None, buf, len(buf)) == R.RBC_ERR_INVALID
    assert L.rbc_step(None, 1) == R.RBC_ERR_INVALID


def test_batch_refuses_invalid_member(R):
    arr = (R.RbcParams * 2)(params(R), params(R, ny=2))
    h = ctypes.c_void_p()
    assert R.lib().rbc_batch_create(arr, 2, ctypes.byref(h)) == R.RBC_ERR_INVALID
    assert h.value is None


def test_valid_case_without_gpu_fails_with_a_status(R):
    # valid parameters on a machine without a GPU: a CUDA error status and a
    # message, not an abort and not a CPU fallback
    h = ctypes.c_void_p()
    rc = R.lib().rbc_create(ctypes.byref(params(R)), ctypes.byref(h))
    if rc == 0:
        R.lib().rbc_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == R.RBC_ERR_CUDA
    assert h.value is None
    assert last_error(R)
