"""rustpde_gb300 -- GB300-native spectral Rayleigh-Benard time step.

Python mirror of rustpde's public interface for the hot path, over the C ABI
of ``libspectral_rbc.so`` (include/spectral_rbc.h):

  * ``Navier2D.new`` / ``Navier2D.new_periodic`` / ``update`` / ``integrate``
    (src/navier/navier.rs, src/lib.rs)
  * ``Space2``, ``Field2`` with ``forward/backward/to_ortho/from_ortho/gradient``
    and the bases ``chebyshev, cheb_dirichlet, cheb_neumann, cheb_dirichlet_bc,
    cheb_neumann_bc, fourier_r2c`` (funspace, src/field.rs)
  * ``Hholtz``, ``HholtzAdi``, ``Poisson`` solvers (src/solver/*.rs)

All numerical work runs in the CUDA library; there is no CPU fallback.  If the
library is not built, every entry point raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libspectral_rbc.so")

RBC_OK = 0
RBC_ERR_INVALID = -1
RBC_ERR_CUDA = -2
RBC_ERR_NUMERIC = -3
RBC_ERR_UNSUPPORTED = -4
RBC_ERR_NOMEM = -5
RBC_ERR_CANCELLED = -6

BOX_ADIABATIC, BOX_CONDUCTING, PERIODIC = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
TEMP, UX, UY, PRES, PSEUDO_PRES, FIELDBC = 0, 1, 2, 3, 4, 5
ADJ_TEMP_RES, ADJ_UX_RES, ADJ_UY_RES = 10, 11, 12
NU, NUVOL, RE, KE, DIV_NORM = 0, 1, 2, 3, 4
CHEBYSHEV, CHEB_DIRICHLET, CHEB_NEUMANN, CHEB_DIRICHLET_BC, CHEB_NEUMANN_BC, FOURIER_R2C = range(6)
HHOLTZ, HHOLTZ_ADI, POISSON = 0, 1, 2

_lock = threading.Lock()
_lib = None


class RbcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class RbcParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("ra", ctypes.c_double), ("pr", ctypes.c_double),
                ("dt", ctypes.c_double), ("aspect", ctypes.c_double), ("kind", ctypes.c_int),
                ("precision", ctypes.c_int)]


_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_SZ = ctypes.c_size_t
CALLBACK = ctypes.CFUNCTYPE(ctypes.c_int, _P, _D, _P)

class RbcServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_active", ctypes.c_int), ("chunk_steps", ctypes.c_int),
                ("setup_threads", ctypes.c_int)]


class RbcRequestResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("status", ctypes.c_int), ("steps", ctypes.c_int),
                ("sim_time", ctypes.c_double), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_done", ctypes.c_double), ("nu", ctypes.c_double), ("ke", ctypes.c_double),
                ("grid_points", ctypes.c_longlong)]


class RbcServerStats(ctypes.Structure):
    _fields_ = [("now", ctypes.c_double), ("pending", ctypes.c_int), ("active", ctypes.c_int),
                ("completed", ctypes.c_longlong), ("bytes_in_use", ctypes.c_size_t),
                ("grid_point_steps", ctypes.c_double), ("steps_launched", ctypes.c_longlong),
                ("rebuilds", ctypes.c_longlong), ("peak_bytes_in_use", ctypes.c_size_t)]


_SIGNATURES = {
    "rbc_last_error": (ctypes.c_char_p, []),
    "rbc_version": (ctypes.c_char_p, []),
    "rbc_create": (_I, [ctypes.POINTER(RbcParams), ctypes.POINTER(_P)]),
    "rbc_destroy": (_I, [_P]),
    "rbc_get_params": (_I, [_P, _DP]),
    "rbc_set_velocity": (_I, [_P, _D, _D, _D]),
    "rbc_set_temperature": (_I, [_P, _D, _D, _D]),
    "rbc_random_disturbance": (_I, [_P, _D, ctypes.c_uint64]),
    "rbc_set_temperature_noise": (_I, [_P, _D, ctypes.c_uint64]),
    "rbc_set_solid": (_I, [_P, _DP, _DP, _SZ]),
    "rbc_get_solid": (_I, [_P, _IP, _DP, _DP, _SZ]),
    "rbc_solid_cylinder_inner": (_I, [_DP, _I, _DP, _I, _D, _D, _D, _DP, _DP]),
    "rbc_solid_roughness_sinusoid": (_I, [_DP, _I, _DP, _I, _D, _D, _DP, _DP]),
    "rbc_solid_porosity": (_I, [_DP, _I, _DP, _I, _D, _D, _DP, _DP]),
    "rbc_solid_porosity_interpolate": (_I, [_I, _I, _D, _D, _DP, _DP]),
    "rbc_step": (_I, [_P, _I]),
    "rbc_synchronize": (_I, [_P]),
    "rbc_get_time": (_I, [_P, _DP]),
    "rbc_set_time": (_I, [_P, _D]),
    "rbc_get_dt": (_I, [_P, _DP]),
    "rbc_status": (_I, [_P, _IP]),
    "rbc_exit": (_I, [_P, _IP]),
    "rbc_integrate": (_I, [_P, _D, _D, CALLBACK, _P, ctypes.POINTER(ctypes.c_long)]),
    "rbc_field_shape": (_I, [_P, _I, _IP, _IP, _IP]),
    "rbc_get_state": (_I, [_P, _I, _DP, _SZ]),
    "rbc_set_state": (_I, [_P, _I, _DP, _SZ]),
    "rbc_get_physical": (_I, [_P, _I, _DP, _SZ]),
    "rbc_get_coords": (_I, [_P, _I, _DP, _DP]),
    "rbc_eval": (_I, [_P, _I, _DP]),
    "rbc_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "rbc_device_bytes": (_I, [_P, ctypes.POINTER(_SZ)]),
    "rbc_profile_step": (_I, [_P, _I, _DP, _I, _IP]),
    "rbc_stage_name": (ctypes.c_char_p, [_P, _I]),
    "rbc_batch_create": (_I, [ctypes.POINTER(RbcParams), _I, ctypes.POINTER(_P)]),
    "rbc_batch_destroy": (_I, [_P]),
    "rbc_batch_size": (_I, [_P, _IP]),
    "rbc_batch_case": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "rbc_batch_step": (_I, [_P, _I]),
    "rbc_batch_synchronize": (_I, [_P]),
    "rbc_batch_layout": (_I, [_P, _IP, _IP]),
    "rbc_batch_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "rbc_batch_state_bytes": (_I, [_P, ctypes.POINTER(_SZ)]),
    "rbc_stats_reset": (_I, [_P]),
    "rbc_stats_update": (_I, [_P]),
    "rbc_stats_info": (_I, [_P, _DP, _DP, ctypes.POINTER(ctypes.c_long)]),
    "rbc_stats_get": (_I, [_P, _I, _DP, _SZ]),
    "rbc_stats_write": (_I, [_P, ctypes.c_char_p]),
    "rbc_diag_record": (_I, [_P]),
    "rbc_diag_series": (_I, [_P, _DP, _DP, _DP, _DP, _I, _IP]),
    "rbc_write_snapshot": (_I, [_P, ctypes.c_char_p]),
    "rbc_read_snapshot": (_I, [_P, ctypes.c_char_p]),
    "rbc_server_create": (_I, [ctypes.POINTER(RbcServerConfig), ctypes.POINTER(_P)]),
    "rbc_server_submit": (_I, [_P, ctypes.POINTER(RbcParams), _D, ctypes.c_uint64, ctypes.POINTER(ctypes.c_longlong)]),
    "rbc_server_poll": (_I, [_P, ctypes.POINTER(RbcRequestResult), _I, _IP]),
    "rbc_server_cancel": (_I, [_P, ctypes.c_longlong, _IP]),
    "rbc_server_wait_idle": (_I, [_P, _D, _IP]),
    "rbc_server_stats": (_I, [_P, ctypes.POINTER(RbcServerStats)]),
    "rbc_server_destroy": (_I, [_P]),
    "rbc_batch_profile_step": (_I, [_P, _I, _DP, _DP, _IP, _I, _IP]),
    "rbc_batch_tuning": (_I, [_P, _I, _IP, _IP, _DP, _DP, _IP]),
    "rbc_batch_tuning_forms": (_I, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "rbc_batch_profile_launches": (_I, [_P, _I, _IP, _IP, _IP, _DP, _DP, _I, _IP]),
    "rbc_stage_bytes": (_I, [_P, _I, _DP]),
    "rbc_kernel_name": (ctypes.c_char_p, [_I]),
    "rbc_batch_state_offset": (_I, [_P, _I, ctypes.POINTER(_SZ)]),
    "rbc_batch_get_state_all": (_I, [_P, _P, _SZ]),
    "rbc_batch_set_state_all": (_I, [_P, _P, _SZ]),
    "rbc_batch_step_io": (_I, [_P, _P, _P, _SZ, _I]),
    "rbc_host_alloc_pinned": (_I, [ctypes.POINTER(_P), _SZ]),
    "rbc_host_free_pinned": (_I, [_P]),
    "rbc_dev_alloc": (_I, [ctypes.POINTER(_P), _SZ]),
    "rbc_dev_free": (_I, [_P]),
    "rbc_memcpy_h2d": (_I, [_P, _P, _SZ]),
    "rbc_memcpy_d2h": (_I, [_P, _P, _SZ]),
    "rbc_device_synchronize": (_I, []),
    "rbc_set_device": (_I, [_I]),
    "rbc_get_device": (_I, [_IP]),
    "fs_space_create": (_I, [_I, _I, _I, _I, ctypes.POINTER(_P)]),
    "fs_space_destroy": (_I, [_P]),
    "fs_space_shape": (_I, [_P, _I, _IP, _IP, _IP]),
    "fs_forward": (_I, [_P, _P, _P, _P]),
    "fs_forward_noalloc": (_I, [_P, _P, _P, _P]),
    "fs_backward": (_I, [_P, _P, _P, _P]),
    "fs_to_ortho": (_I, [_P, _P, _P, _P]),
    "fs_from_ortho": (_I, [_P, _P, _P, _P]),
    "fs_gradient": (_I, [_P, _P, _P, _I, _I, _DP, _P]),
    "fs_lanes_create": (_I, [_I, _I, _I, ctypes.POINTER(_P)]),
    "fs_lanes_destroy": (_I, [_P]),
    "fs_lanes_shape": (_I, [_P, _IP, _IP]),
    "fs_lanes_set_hholtz": (_I, [_P, _D]),
    "fs_lanes_apply": (_I, [_P, _I, _P, _P, _I, _P]),
    "fs_lanes_status": (_I, [_P, _P, ctypes.POINTER(ctypes.c_uint)]),
    "rbc_set_gemm_wait_limit": (_I, [ctypes.c_longlong]),
    "rbc_adjoint_create": (_I, [ctypes.POINTER(RbcParams), ctypes.POINTER(_P)]),
    "rbc_adjoint_destroy": (_I, [_P]),
    "rbc_adjoint_set_velocity": (_I, [_P, _D, _D, _D]),
    "rbc_adjoint_set_temperature": (_I, [_P, _D, _D, _D]),
    "rbc_adjoint_step": (_I, [_P, _I]),
    "rbc_adjoint_synchronize": (_I, [_P]),
    "rbc_adjoint_get_time": (_I, [_P, _DP]),
    "rbc_adjoint_set_time": (_I, [_P, _D]),
    "rbc_adjoint_field_shape": (_I, [_P, _I, _IP, _IP, _IP]),
    "rbc_adjoint_get_state": (_I, [_P, _I, _DP, _SZ]),
    "rbc_adjoint_set_state": (_I, [_P, _I, _DP, _SZ]),
    "rbc_adjoint_eval": (_I, [_P, _I, _DP]),
    "rbc_adjoint_residual": (_I, [_P, _DP]),
    "rbc_adjoint_exit": (_I, [_P, _IP]),
    "rbc_adjoint_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "rbc_adjoint_write_snapshot": (_I, [_P, ctypes.c_char_p]),
    "rbc_adjoint_read_snapshot": (_I, [_P, ctypes.c_char_p]),
    "df_create": (_I, [_I, _I, _I, _I, _D, _D, ctypes.POINTER(_P)]),
    "df_destroy": (_I, [_P]),
    "df_shape": (_I, [_P, _I, _IP, _IP, _IP]),
    "df_get_state": (_I, [_P, _DP, _SZ]),
    "df_set_state": (_I, [_P, _DP, _SZ]),
    "df_impulse": (_I, [_P]),
    "df_add_force": (_I, [_P, _DP, _SZ]),
    "df_add_fieldbc": (_I, [_P, _I, _I, _DP, _SZ]),
    "df_step": (_I, [_P, _I]),
    "df_synchronize": (_I, [_P]),
    "df_get_time": (_I, [_P, _DP]),
    "df_get_dt": (_I, [_P, _DP]),
    "df_get_physical": (_I, [_P, _I, _DP, _SZ]),
    "df_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "sv_create": (_I, [_P, _I, _DP, ctypes.POINTER(_P)]),
    "sv_destroy": (_I, [_P]),
    "sv_solve": (_I, [_P, _P, _P, _P]),
}


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with python -m rustpde_gb300.build "
                                   "(there is no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _check(rc):
    if rc != RBC_OK:
        raise RbcError(rc, lib().rbc_last_error().decode())


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


# ---------------------------------------------------------------------------
# device buffers (plain cudaMalloc through the C ABI)
# ---------------------------------------------------------------------------
class PinnedArray:
    """A numpy view of page-locked host memory (cudaHostAlloc)."""

    def __init__(self, shape, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * self.dtype.itemsize
        p = _P()
        _check(lib().rbc_host_alloc_pinned(ctypes.byref(p), max(n, 16)))
        self.ptr = p
        buf = (ctypes.c_char * max(n, 16)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        p = getattr(self, "ptr", None)
        if p is not None and _lib is not None:
            self.array = None
            _lib.rbc_host_free_pinned(p)
            self.ptr = None


class DeviceArray:
    """A device array of float64 / complex128 values."""

    def __init__(self, shape, complex_=False):
        self.shape = tuple(int(s) for s in shape)
        self.complex = bool(complex_)
        self.nbytes = int(np.prod(self.shape)) * (16 if complex_ else 8)
        p = _P()
        _check(lib().rbc_dev_alloc(ctypes.byref(p), max(self.nbytes, 16)))
        self.ptr = p

    @classmethod
    def from_host(cls, a):
        a = np.ascontiguousarray(a)
        cx = np.iscomplexobj(a)
        a = a.astype(np.complex128 if cx else np.float64, copy=False)
        d = cls(a.shape, cx)
        _check(lib().rbc_memcpy_h2d(d.ptr, a.ctypes.data_as(_P), d.nbytes))
        return d

    def to_host(self):
        out = np.empty(self.shape, dtype=np.complex128 if self.complex else np.float64)
        _check(lib().rbc_memcpy_d2h(out.ctypes.data_as(_P), self.ptr, self.nbytes))
        return out

    def __del__(self):
        p = getattr(self, "ptr", None)
        if p is not None and _lib is not None:
            _lib.rbc_dev_free(p)
            self.ptr = None


# ---------------------------------------------------------------------------
# funspace: bases, Space2, Field2
# ---------------------------------------------------------------------------
class Base:
    def __init__(self, kind, n):
        self.kind = int(kind)
        self.n = int(n)


def chebyshev(n):
    return Base(CHEBYSHEV, n)


def cheb_dirichlet(n):
    return Base(CHEB_DIRICHLET, n)


def cheb_neumann(n):
    return Base(CHEB_NEUMANN, n)


def cheb_dirichlet_bc(n):
    return Base(CHEB_DIRICHLET_BC, n)


def cheb_neumann_bc(n):
    return Base(CHEB_NEUMANN_BC, n)


def fourier_r2c(n):
    return Base(FOURIER_R2C, n)


class Space2:
    """Space2::new(base0, base1) (funspace/src/space2.rs)."""

    def __init__(self, base0: Base, base1: Base):
        h = _P()
        _check(lib().fs_space_create(base0.kind, base0.n, base1.kind, base1.n, ctypes.byref(h)))
        self._h = h
        self.base0, self.base1 = base0, base1
        self.physical = self._shape(0)[:2]
        sp = self._shape(1)
        self.spectral = sp[:2]
        self.is_complex = bool(sp[2])
        self.ortho = self._shape(2)[:2]

    def _shape(self, which):
        a, b, c = _I(), _I(), _I()
        _check(lib().fs_space_shape(self._h, which, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.fs_space_destroy(h)
            self._h = None

    # device-buffer level (drop-in primitives)
    def forward_dev(self, d_phys, d_spec, stream=None):
        _check(lib().fs_forward(self._h, d_phys.ptr, d_spec.ptr, stream))

    def forward_noalloc_dev(self, d_phys, d_spec, stream=None):
        """forward_dev through fs_forward_noalloc: no allocation; the
        intermediate uses the library's fixed device scratch, shared by all
        calls on the device (calls that may overlap in time race on it)."""
        _check(lib().fs_forward_noalloc(self._h, d_phys.ptr, d_spec.ptr, stream))

    def backward_dev(self, d_spec, d_phys, stream=None):
        _check(lib().fs_backward(self._h, d_spec.ptr, d_phys.ptr, stream))

    def to_ortho_dev(self, d_spec, d_ortho, stream=None):
        _check(lib().fs_to_ortho(self._h, d_spec.ptr, d_ortho.ptr, stream))

    def from_ortho_dev(self, d_ortho, d_spec, stream=None):
        _check(lib().fs_from_ortho(self._h, d_ortho.ptr, d_spec.ptr, stream))

    def gradient_dev(self, d_spec, d_ortho, deriv, scale=None, stream=None):
        sc = None
        if scale is not None:
            self._sc = np.asarray(scale, dtype=np.float64)
            sc = _dptr(self._sc)
        _check(lib().fs_gradient(self._h, d_spec.ptr, d_ortho.ptr, int(deriv[0]), int(deriv[1]), sc, stream))

    # host-array convenience (copies in and out)
    def _run(self, fn, a, out_shape, out_complex, *args):
        d_in = DeviceArray.from_host(a)
        d_out = DeviceArray(out_shape, out_complex)
        fn(d_in, d_out, *args)
        _check(lib().rbc_device_synchronize())
        return d_out.to_host()

    def forward(self, v):
        return self._run(self.forward_dev, np.asarray(v, dtype=np.float64), self.spectral, self.is_complex)

    def backward(self, vhat):
        return self._run(self.backward_dev, self._spec(vhat), self.physical, False)

    def to_ortho(self, vhat):
        return self._run(self.to_ortho_dev, self._spec(vhat), self.ortho, self.is_complex)

    def from_ortho(self, o):
        return self._run(self.from_ortho_dev, self._spec(o), self.spectral, self.is_complex)

    def gradient(self, vhat, deriv, scale=None):
        return self._run(self.gradient_dev, self._spec(vhat), self.ortho, self.is_complex, deriv, scale)

    def _spec(self, a):
        return np.asarray(a, dtype=np.complex128 if self.is_complex else np.float64)


class Field2:
    """Field2 (src/field.rs:67-129): physical ``v`` and spectral ``vhat``."""

    def __init__(self, space: Space2):
        self.space = space
        self.v = np.zeros(space.physical)
        self.vhat = np.zeros(space.spectral, dtype=np.complex128 if space.is_complex else np.float64)

    def forward(self):
        self.vhat = self.space.forward(self.v)

    def backward(self):
        self.v = self.space.backward(self.vhat)

    def to_ortho(self):
        return self.space.to_ortho(self.vhat)

    def from_ortho(self, o):
        self.vhat = self.space.from_ortho(o)

    def gradient(self, deriv, scale=None):
        return self.space.gradient(self.vhat, deriv, scale)


class Navier2DAdjoint:
    """Navier2DAdjoint (src/navier/navier_adjoint.rs): adjoint descent towards
    a steady state of the Rayleigh-Benard equations, on the GPU.  ``dt`` is the
    pseudo time step; each update runs one Navier2D step of dt = 1e-2."""

    def __init__(self, nx, ny, ra, pr, dt, aspect, kind):
        p = RbcParams(int(nx), int(ny), float(ra), float(pr), float(dt), float(aspect), int(kind), PREC_FP64)
        h = _P()
        _check(lib().rbc_adjoint_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        self.nx, self.ny, self.kind, self.dt = int(nx), int(ny), int(kind), float(dt)

    @classmethod
    def new(cls, nx, ny, ra, pr, dt, aspect, adiabatic=True):
        return cls(nx, ny, ra, pr, dt, aspect, BOX_ADIABATIC if adiabatic else BOX_CONDUCTING)

    @classmethod
    def new_periodic(cls, nx, ny, ra, pr, dt, aspect):
        return cls(nx, ny, ra, pr, dt, aspect, PERIODIC)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.rbc_adjoint_destroy(h)
            self._h = None

    def set_velocity(self, amp, m, n):
        _check(lib().rbc_adjoint_set_velocity(self._h, float(amp), float(m), float(n)))

    def set_temperature(self, amp, m, n):
        _check(lib().rbc_adjoint_set_temperature(self._h, float(amp), float(m), float(n)))

    def update(self, nsteps: int = 1):
        _check(lib().rbc_adjoint_step(self._h, int(nsteps)))

    def synchronize(self):
        _check(lib().rbc_adjoint_synchronize(self._h))

    def get_time(self):
        t = _D()
        _check(lib().rbc_adjoint_get_time(self._h, ctypes.byref(t)))
        return t.value

    def get_dt(self):
        return self.dt

    def reset_time(self):
        _check(lib().rbc_adjoint_set_time(self._h, 0.0))

    def shape(self, field):
        a, b, c = _I(), _I(), _I()
        _check(lib().rbc_adjoint_field_shape(self._h, field, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return (a.value, b.value), bool(c.value)

    def get(self, field):
        sh, cx = self.shape(field)
        out = np.empty(sh, dtype=np.complex128 if cx else np.float64)
        _check(lib().rbc_adjoint_get_state(self._h, field, out.ctypes.data_as(_DP), out.size * (2 if cx else 1)))
        return out

    def set(self, field, arr):
        sh, cx = self.shape(field)
        a = np.ascontiguousarray(arr, dtype=np.complex128 if cx else np.float64)
        if a.shape != sh:
            raise ValueError(f"shape mismatch: got {a.shape}, expected {sh}")
        _check(lib().rbc_adjoint_set_state(self._h, field, a.ctypes.data_as(_DP), a.size * (2 if cx else 1)))

    def eval(self, what):
        v = _D()
        _check(lib().rbc_adjoint_eval(self._h, what, ctypes.byref(v)))
        return v.value

    def eval_nu(self):
        return self.eval(NU)

    def eval_nuvol(self):
        return self.eval(NUVOL)

    def eval_re(self):
        return self.eval(RE)

    def residual(self):
        """L2 norms (u, v, T) of the unsmoothed and of the smoothed residual."""
        out = np.zeros(6)
        _check(lib().rbc_adjoint_residual(self._h, _dptr(out)))
        return out

    def callback(self):
        """The diagnostics Navier2DAdjoint::callback prints and logs
        (navier_adjoint.rs:811-886), returned instead of written."""
        r = self.residual()
        return {"time": self.get_time(), "div": self.eval(DIV_NORM), "Nu": self.eval_nu(),
                "Nuvol": self.eval_nuvol(), "Re": self.eval_re(), "res_unsmoothed": float(r[:3].sum()),
                "res_smoothed": float(r[3:].sum())}

    def exit(self):
        s = _I()
        _check(lib().rbc_adjoint_exit(self._h, ctypes.byref(s)))
        return bool(s.value)

    def stream(self):
        s = _P()
        _check(lib().rbc_adjoint_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def write(self, filename):
        """Navier2DAdjoint::write (navier_adjoint.rs:1005-1040)."""
        _check(lib().rbc_adjoint_write_snapshot(self._h, filename.encode()))

    def read(self, filename):
        """Navier2DAdjoint::read (navier_adjoint.rs:991-999): temp, ux, uy, time."""
        _check(lib().rbc_adjoint_read_snapshot(self._h, filename.encode()))


class Diffusion2D:
    """Diffusion2D (src/navier/diffusion.rs:113-238): the fully implicit 2-D
    diffusion equation on the field's space, stepped on the GPU (df_* of the
    C library).  ``Diffusion2D(field, kappa, dt)`` takes the field's space and
    its current ``vhat`` as the initial state."""

    def __init__(self, field: Field2, kappa, dt):
        sp = field.space
        h = _P()
        _check(lib().df_create(sp.base0.kind, sp.base0.n, sp.base1.kind, sp.base1.n, float(kappa), float(dt),
                               ctypes.byref(h)))
        self._h = h
        self.space = sp
        self.kappa, self.dt = float(kappa), float(dt)
        self._fieldbc = None
        self.set_state(field.vhat)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.df_destroy(h)
            self._h = None

    def _cplx(self):
        return np.complex128 if self.space.is_complex else np.float64

    def get_state(self):
        out = np.empty(self.space.spectral, dtype=self._cplx())
        _check(lib().df_get_state(self._h, out.ctypes.data_as(_DP), out.size * (2 if self.space.is_complex else 1)))
        return out

    def set_state(self, vhat):
        a = np.ascontiguousarray(vhat, dtype=self._cplx())
        if a.shape != tuple(self.space.spectral):
            raise ValueError(f"shape mismatch: got {a.shape}, expected {self.space.spectral}")
        _check(lib().df_set_state(self._h, a.ctypes.data_as(_DP), a.size * (2 if self.space.is_complex else 1)))

    @property
    def vhat(self):
        return self.get_state()

    def impulse(self):
        """diffusion.rs:156-163: unit impulse at (n/2, m/2), forward transform."""
        _check(lib().df_impulse(self._h))

    def add_force(self, force):
        """diffusion.rs:168-171 (force with field.v's shape)."""
        f = np.ascontiguousarray(force, dtype=np.float64)
        if f.shape != tuple(self.space.physical):
            raise ValueError(f"shape mismatch: got {f.shape}, expected {self.space.physical}")
        _check(lib().df_add_force(self._h, _dptr(f), f.size))

    def add_fieldbc(self, fieldbc: Field2):
        """diffusion.rs:176-179: inhomogeneous boundary field (its vhat)."""
        sp = fieldbc.space
        if tuple(sp.physical) != tuple(self.space.physical):
            raise ValueError("shape mismatch between the field and the boundary field")
        a = np.ascontiguousarray(fieldbc.vhat, dtype=np.complex128 if sp.is_complex else np.float64)
        _check(lib().df_add_fieldbc(self._h, sp.base0.kind, sp.base1.kind, a.ctypes.data_as(_DP),
                                    a.size * (2 if sp.is_complex else 1)))
        self._fieldbc = fieldbc

    def update(self, nsteps: int = 1):
        """Integrate::update (diffusion.rs:186-207), nsteps times (asynchronous)."""
        _check(lib().df_step(self._h, int(nsteps)))

    def synchronize(self):
        _check(lib().df_synchronize(self._h))

    def get_time(self):
        t = _D()
        _check(lib().df_get_time(self._h, ctypes.byref(t)))
        return t.value

    def get_dt(self):
        return self.dt

    def get_physical(self, with_bc=False):
        out = np.empty(self.space.physical)
        _check(lib().df_get_physical(self._h, int(bool(with_bc)), _dptr(out), out.size))
        return out

    def callback(self):
        """The physical field as Diffusion2D::callback writes it (with the
        boundary field added, diffusion.rs:214-225), returned instead of written."""
        return self.get_physical(with_bc=True)

    def stream(self):
        s = _P()
        _check(lib().df_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def exit(self):
        return False


OP_FORWARD, OP_BACKWARD, OP_TO_ORTHO, OP_FROM_ORTHO, OP_HHOLTZ = 0, 1, 2, 3, 4


class Lanes:
    """Batched 1-D operations of one Chebyshev-family basis on many lanes
    (row-major lanes x length): forward / backward / to_ortho / from_ortho and
    the 1-D HholtzAdi solve, in FP64 or mixed precision (tensor-core 3xTF32
    dense products, FP64 banded sweep)."""

    def __init__(self, base: Base, precision=PREC_FP64, hholtz_c=None):
        h = _P()
        _check(lib().fs_lanes_create(base.kind, base.n, int(precision), ctypes.byref(h)))
        self._h = h
        n, m = _I(), _I()
        _check(lib().fs_lanes_shape(h, ctypes.byref(n), ctypes.byref(m)))
        self.n, self.m = n.value, m.value
        if hholtz_c is not None:
            _check(lib().fs_lanes_set_hholtz(h, float(hholtz_c)))

    def lengths(self, op):
        return {OP_FORWARD: (self.n, self.m), OP_BACKWARD: (self.m, self.n), OP_TO_ORTHO: (self.m, self.n),
                OP_FROM_ORTHO: (self.n, self.m), OP_HHOLTZ: (self.n, self.m)}[op]

    def apply_dev(self, op, d_in, d_out, lanes, stream=None):
        _check(lib().fs_lanes_apply(self._h, int(op), d_in.ptr, d_out.ptr, int(lanes), stream))

    def status(self, stream=None):
        """Wait for `stream` and return (and clear) the status word of the
        applies so far: bit 1 when a tensor-core completion wait timed out."""
        v = ctypes.c_uint()
        _check(lib().fs_lanes_status(self._h, stream, ctypes.byref(v)))
        return v.value

    def apply(self, op, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        il, ol = self.lengths(op)
        assert a.shape[-1] == il
        lanes = a.size // il
        d_in = DeviceArray.from_host(a)
        d_out = DeviceArray((lanes, ol))
        self.apply_dev(op, d_in, d_out, lanes)
        _check(lib().rbc_device_synchronize())
        return d_out.to_host()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.fs_lanes_destroy(h)
            self._h = None


class _Solver:
    kind = HHOLTZ

    def __init__(self, field_or_space, c):
        space = field_or_space.space if isinstance(field_or_space, Field2) else field_or_space
        self.space = space
        self._c = np.asarray(c, dtype=np.float64).reshape(2)
        h = _P()
        _check(lib().sv_create(space._h, self.kind, _dptr(self._c), ctypes.byref(h)))
        self._h = h

    def solve_dev(self, d_in, d_out, stream=None):
        _check(lib().sv_solve(self._h, d_in.ptr, d_out.ptr, stream))

    def solve(self, rhs):
        rhs = np.asarray(rhs, dtype=np.complex128 if self.space.is_complex else np.float64)
        d_in = DeviceArray.from_host(rhs)
        d_out = DeviceArray(self.space.spectral, self.space.is_complex)
        self.solve_dev(d_in, d_out)
        _check(lib().rbc_device_synchronize())
        return d_out.to_host()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.sv_destroy(h)
            self._h = None


class Hholtz(_Solver):
    """Hholtz::new (src/solver/hholtz.rs:42-76)."""
    kind = HHOLTZ


class HholtzAdi(_Solver):
    """HholtzAdi::new (src/solver/hholtz_adi.rs:44-63)."""
    kind = HHOLTZ_ADI


class Poisson(_Solver):
    """Poisson::new (src/solver/poisson.rs:50-90)."""
    kind = POISSON


# ---------------------------------------------------------------------------
# Navier2D
# ---------------------------------------------------------------------------
class Navier2D:
    """Navier2D (src/navier/navier.rs) on the GPU.

    ``Navier2D.new(nx, ny, ra, pr, dt, aspect, adiabatic)`` and
    ``Navier2D.new_periodic(nx, ny, ra, pr, dt, aspect)`` mirror the reference
    constructors, including the initial ``random_disturbance(0.1)``, which is
    seeded here (``seed``) where the reference draws from an unseeded RNG.
    """

    def __init__(self, nx, ny, ra, pr, dt, aspect, kind, precision=PREC_FP64, seed=None, _borrowed=None):
        if _borrowed is not None:
            h = _P(_borrowed)
            self._borrowed = True
        else:
            p = RbcParams(int(nx), int(ny), float(ra), float(pr), float(dt), float(aspect), int(kind), int(precision))
            h = _P()
            _check(lib().rbc_create(ctypes.byref(p), ctypes.byref(h)))
            self._borrowed = False
        self._h = h
        self.kind = kind
        self.periodic = kind == PERIODIC
        self.nx, self.ny = int(nx), int(ny)
        pv = np.zeros(7)
        _check(lib().rbc_get_params(h, _dptr(pv)))
        self.nu, self.ka, self.ra, self.pr, self.dt = (float(x) for x in pv[:5])
        self.scale = pv[5:7].copy()
        if seed is not None:
            self.random_disturbance(0.1, seed)

    @classmethod
    def new(cls, nx, ny, ra, pr, dt, aspect, adiabatic=True, seed=0):
        return cls(nx, ny, ra, pr, dt, aspect, BOX_ADIABATIC if adiabatic else BOX_CONDUCTING, seed=seed)

    @classmethod
    def new_periodic(cls, nx, ny, ra, pr, dt, aspect, seed=0):
        return cls(nx, ny, ra, pr, dt, aspect, PERIODIC, seed=seed)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None and not getattr(self, "_borrowed", False):
            _lib.rbc_destroy(h)
        self._h = None

    # --- Integrate trait (src/lib.rs:135-146)
    def update(self, nsteps: int = 1):
        _check(lib().rbc_step(self._h, int(nsteps)))

    def synchronize(self):
        _check(lib().rbc_synchronize(self._h))

    def get_time(self):
        t = _D()
        _check(lib().rbc_get_time(self._h, ctypes.byref(t)))
        return t.value

    @property
    def time(self):
        return self.get_time()

    def get_dt(self):
        return self.dt

    def reset_time(self):
        _check(lib().rbc_set_time(self._h, 0.0))

    def exit(self):
        s = _I()
        _check(lib().rbc_exit(self._h, ctypes.byref(s)))
        return bool(s.value)

    def status(self):
        s = _I()
        _check(lib().rbc_status(self._h, ctypes.byref(s)))
        return s.value

    def callback(self):
        """Diagnostics of Navier2D::callback (navier.rs:775-853) without file I/O."""
        return {"time": self.get_time(), "div": self.eval(DIV_NORM), "Nu": self.eval_nu(), "Nuvol": self.eval_nuvol(),
                "Re": self.eval_re()}

    # --- initial conditions
    def set_velocity(self, amp, m, n):
        _check(lib().rbc_set_velocity(self._h, float(amp), float(m), float(n)))

    def set_temperature(self, amp, m, n):
        _check(lib().rbc_set_temperature(self._h, float(amp), float(m), float(n)))

    def random_disturbance(self, amp, seed=0):
        _check(lib().rbc_random_disturbance(self._h, float(amp), ctypes.c_uint64(seed)))

    def set_temperature_noise(self, amp, seed):
        _check(lib().rbc_set_temperature_noise(self._h, float(amp), ctypes.c_uint64(seed)))

    def zero_pressure(self):
        for f in (PRES, PSEUDO_PRES):
            self.set(f, np.zeros_like(self.get(f)))

    # --- solid obstacles (navier.rs:189-190 `pub solid: Option<[Array2<f64>; 2]>`)
    @property
    def solid(self):
        """None, or [mask, value] (physical nx x ny arrays)."""
        present = _I()
        _check(lib().rbc_get_solid(self._h, ctypes.byref(present), None, None, 0))
        if not present.value:
            return None
        m, v = np.empty((self.nx, self.ny)), np.empty((self.nx, self.ny))
        _check(lib().rbc_get_solid(self._h, ctypes.byref(present), _dptr(m), _dptr(v), m.size))
        return [m, v]

    @solid.setter
    def solid(self, mv):
        if mv is None:
            _check(lib().rbc_set_solid(self._h, None, None, 0))
            return
        m = np.ascontiguousarray(mv[0], dtype=np.float64)
        v = np.ascontiguousarray(mv[1], dtype=np.float64)
        if m.shape != (self.nx, self.ny) or v.shape != m.shape:
            raise ValueError(f"solid mask and value must have shape {(self.nx, self.ny)}")
        _check(lib().rbc_set_solid(self._h, _dptr(m), _dptr(v), m.size))

    # --- state
    def shape(self, field):
        a, b, c = _I(), _I(), _I()
        _check(lib().rbc_field_shape(self._h, field, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return (a.value, b.value), bool(c.value)

    def get(self, field):
        sh, cx = self.shape(field)
        out = np.empty(sh, dtype=np.complex128 if cx else np.float64)
        _check(lib().rbc_get_state(self._h, field, out.ctypes.data_as(_DP), out.size * (2 if cx else 1)))
        return out

    def set(self, field, arr):
        sh, cx = self.shape(field)
        a = np.ascontiguousarray(arr, dtype=np.complex128 if cx else np.float64)
        if a.shape != sh:
            raise ValueError(f"shape mismatch: got {a.shape}, expected {sh}")
        _check(lib().rbc_set_state(self._h, field, a.ctypes.data_as(_DP), a.size * (2 if cx else 1)))

    def get_physical(self, field):
        out = np.empty((self.nx, self.ny))
        _check(lib().rbc_get_physical(self._h, field, _dptr(out), out.size))
        return out

    def coords(self, field=UX):
        """Grid coordinates (x, y) of a field, scaled like Navier2D::_scale."""
        x, y = np.zeros(self.nx), np.zeros(self.ny)
        _check(lib().rbc_get_coords(self._h, field, _dptr(x), _dptr(y)))
        return x, y

    # --- diagnostics
    def eval(self, what):
        v = _D()
        _check(lib().rbc_eval(self._h, what, ctypes.byref(v)))
        return v.value

    def eval_nu(self):
        return self.eval(NU)

    def eval_nuvol(self):
        return self.eval(NUVOL)

    def eval_re(self):
        return self.eval(RE)

    def eval_ke(self):
        return self.eval(KE)

    def div_norm(self):
        return self.eval(DIV_NORM)

    # --- statistics (statistics.rs) and the callback's diagnostics series
    def stats_reset(self):
        _check(lib().rbc_stats_reset(self._h))

    def stats_update(self):
        _check(lib().rbc_stats_update(self._h))

    def stats_info(self):
        t, a, n = _D(), _D(), ctypes.c_long()
        _check(lib().rbc_stats_info(self._h, ctypes.byref(t), ctypes.byref(a), ctypes.byref(n)))
        return {"tot_time": t.value, "avg_time": a.value, "num_save": n.value}

    def stats_get(self, which):
        """which: 0 temperature average, 1 ux, 2 uy, 3 Nusselt field (spectral, field space)."""
        sh, cx = self.shape(FIELDBC)
        shape = (sh[0], self.ny)
        out = np.empty(shape, dtype=np.complex128 if cx else np.float64)
        _check(lib().rbc_stats_get(self._h, int(which), out.ctypes.data_as(_DP), out.size * (2 if cx else 1)))
        return out

    def stats_write(self, filename):
        _check(lib().rbc_stats_write(self._h, os.fsencode(filename)))

    def diag_record(self):
        _check(lib().rbc_diag_record(self._h))

    def diag_series(self):
        n = _I()
        _check(lib().rbc_diag_series(self._h, None, None, None, None, 0, ctypes.byref(n)))
        arrs = [np.zeros(n.value) for _ in range(4)]
        _check(lib().rbc_diag_series(self._h, *[_dptr(a) for a in arrs], n.value, ctypes.byref(n)))
        return dict(zip(("time", "nu", "nuvol", "re"), arrs))

    def write(self, filename):
        """Navier2D::write (navier.rs:975-1013): snapshot file + JSON sidecar."""
        _check(lib().rbc_write_snapshot(self._h, os.fsencode(filename)))

    def read(self, filename):
        """Navier2D::read (navier.rs:961-972): restore fields and time
        (broadcast from another resolution)."""
        _check(lib().rbc_read_snapshot(self._h, os.fsencode(filename)))

    def profile_step(self, nsteps=10, with_bytes=False):
        """Mean device time (ms) of each kernel of the step, summed over the
        stages that run the same kernel: {kernel name: ms}, or {name: (ms,
        algorithmic bytes)} with ``with_bytes``."""
        ms = np.zeros(64)
        n = _I()
        _check(lib().rbc_profile_step(self._h, int(nsteps), _dptr(ms), 64, ctypes.byref(n)))
        out = {}
        for k in range(n.value):
            name = lib().rbc_stage_name(self._h, k).decode()
            b = _D()
            _check(lib().rbc_stage_bytes(self._h, k, ctypes.byref(b)))
            t, by = out.get(name, (0.0, 0.0))
            out[name] = (t + float(ms[k]), by + b.value)
        return out if with_bytes else {k: v[0] for k, v in out.items()}

    def stream(self):
        s = _P()
        _check(lib().rbc_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def device_bytes(self):
        b = _SZ()
        _check(lib().rbc_device_bytes(self._h, ctypes.byref(b)))
        return b.value


class Batch:
    """Independent cases advanced together (rbc_batch_*).  ``params`` is a
    list of (nx, ny, ra, pr, dt, aspect, kind[, precision]) tuples;
    ``precision`` (default for all) applies to tuples without one.
    ``cases[i]`` is a borrowed Navier2D handle of case i (initial conditions,
    state, diagnostics)."""

    def __init__(self, params, precision=PREC_FP64):
        full = [tuple(p) if len(p) == 8 else tuple(p) + (precision,) for p in params]
        arr = (RbcParams * len(full))()
        for i, (nx, ny, ra, pr, dt, asp, kind, prec) in enumerate(full):
            arr[i] = RbcParams(int(nx), int(ny), float(ra), float(pr), float(dt), float(asp), int(kind), int(prec))
        h = _P()
        _check(lib().rbc_batch_create(arr, len(full), ctypes.byref(h)))
        self._h = h
        self.cases = []
        for i, (nx, ny, ra, pr, dt, asp, kind, prec) in enumerate(full):
            c = _P()
            _check(lib().rbc_batch_case(h, i, ctypes.byref(c)))
            self.cases.append(Navier2D(nx, ny, ra, pr, dt, asp, kind, prec, _borrowed=c.value))

    def update(self, nsteps=1):
        _check(lib().rbc_batch_step(self._h, int(nsteps)))

    def synchronize(self):
        _check(lib().rbc_batch_synchronize(self._h))

    def layout(self):
        a, b = _I(), _I()
        _check(lib().rbc_batch_layout(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def stream(self):
        s = _P()
        _check(lib().rbc_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def profile_step(self, nsteps=5):
        """{kernel name: (mean ms per step, algorithmic bytes per step)} with
        every launch timed alone (advances the batch by nsteps steps)."""
        cap = 64
        ms = (ctypes.c_double * cap)()
        by = (ctypes.c_double * cap)()
        kd = (ctypes.c_int * cap)()
        n = _I()
        _check(lib().rbc_batch_profile_step(self._h, int(nsteps), ms, by, kd, cap, ctypes.byref(n)))
        return {lib().rbc_kernel_name(kd[k]).decode(): (ms[k], by[k]) for k in range(n.value)}

    def profile_launches(self, nsteps=3):
        """[(bucket, pass, kernel name, mean ms, algorithmic bytes)] for every
        launch of the step, each timed alone (advances the batch by nsteps)."""
        cap = 256
        kd, bk, ps = (ctypes.c_int * cap)(), (ctypes.c_int * cap)(), (ctypes.c_int * cap)()
        ms, by = (ctypes.c_double * cap)(), (ctypes.c_double * cap)()
        n = _I()
        _check(lib().rbc_batch_profile_launches(self._h, int(nsteps), kd, bk, ps, ms, by, cap, ctypes.byref(n)))
        return [(bk[k], ps[k], lib().rbc_kernel_name(kd[k]).decode(), ms[k], by[k]) for k in range(min(n.value, cap))]

    def tuning(self):
        """Autotuner decisions: [(pass, ms one CTA per lane, ms one thread per lane, chosen)]."""
        n = _I()
        _check(lib().rbc_batch_tuning(self._h, -1, None, None, None, None, ctypes.byref(n)))
        out = []
        for k in range(n.value):
            a, b, ta, tb = _I(), _I(), _D(), _D()
            _check(lib().rbc_batch_tuning(self._h, k, ctypes.byref(a), ctypes.byref(b), ctypes.byref(ta),
                                          ctypes.byref(tb), ctypes.byref(n)))
            out.append((lib().rbc_kernel_name(a.value).decode(), ta.value, tb.value,
                        "lanes" if tb.value < ta.value else "cta"))
        return out

    def tuning_forms(self):
        """The forms the autotuner kept, as the RBC_BATCH_FORM string: the FP64
        passes' digits, then after a ';' the GEMM passes' ("2,0,...;0,0,...")."""
        buf = ctypes.create_string_buffer(256)
        _check(lib().rbc_batch_tuning_forms(self._h, buf, len(buf)))
        return buf.value.decode()

    def state_bytes(self):
        n = _SZ()
        _check(lib().rbc_batch_state_bytes(self._h, ctypes.byref(n)))
        return n.value

    def get_state_all(self, host):
        """Copy every case's spectral state into ``host`` (a uint8 array of
        state_bytes(), e.g. PinnedArray(...).array)."""
        _check(lib().rbc_batch_get_state_all(self._h, host.ctypes.data_as(_P), host.nbytes))

    def set_state_all(self, host):
        _check(lib().rbc_batch_set_state_all(self._h, host.ctypes.data_as(_P), host.nbytes))

    def state_offset(self, i):
        n = _SZ()
        _check(lib().rbc_batch_state_offset(self._h, int(i), ctypes.byref(n)))
        return n.value

    def step_io(self, host_in, host_out, nsteps=1):
        """set_state_all(host_in), update(nsteps), get_state_all(host_out) in
        one call, each group's copies overlapping the other groups' steps
        (rbc_batch_step_io); returns when host_out is written."""
        if host_in.nbytes != host_out.nbytes:
            raise ValueError("step_io: host_in and host_out differ in size")
        _check(lib().rbc_batch_step_io(self._h, host_in.ctypes.data_as(_P), host_out.ctypes.data_as(_P),
                                       host_in.nbytes, int(nsteps)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            for c in getattr(self, "cases", []):
                c._h = None
            _lib.rbc_batch_destroy(h)
            self._h = None


class Server:
    """Serving loop (rbc_server_*): requests are RBC solves (params, horizon
    in time units, initial-condition seed) admitted against a device-memory
    budget and advanced together with continuous batching."""

    def __init__(self, hbm_budget_bytes=150 * 10**9, max_active=256, chunk_steps=8, setup_threads=4):
        cfg = RbcServerConfig(int(hbm_budget_bytes), int(max_active), int(chunk_steps), int(setup_threads))
        h = _P()
        _check(lib().rbc_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        # id -> (params, horizon, seed) of the requests whose results poll()
        # has not returned yet; poll() moves them into the results
        self._requests = {}

    def submit(self, params, horizon, seed, precision=PREC_FP64):
        nx, ny, ra, pr, dt, asp, kind = params[:7]
        prec = params[7] if len(params) > 7 else precision
        p = RbcParams(int(nx), int(ny), float(ra), float(pr), float(dt), float(asp), int(kind), int(prec))
        rid = ctypes.c_longlong()
        _check(lib().rbc_server_submit(self._h, ctypes.byref(p), float(horizon), int(seed), ctypes.byref(rid)))
        self._requests[rid.value] = ((int(nx), int(ny), float(ra), float(pr), float(dt), float(asp), int(kind),
                                      int(prec)), float(horizon), int(seed))
        return rid.value

    def record(self, result):
        """One request's record for a JSON-lines log: id, sizes and parameters,
        horizon, seed, status, steps, simulated time, wall time from submission
        to result (and the part spent queued and in set-up), Nu and KE."""
        req = result.get("request") or self._requests.get(result["id"], ((None,) * 8, None, None))
        p, horizon, seed = req
        keys = ("nx", "ny", "ra", "pr", "dt", "aspect", "kind", "precision")
        rec = {"id": result["id"], **dict(zip(keys, p)), "horizon": horizon, "seed": seed,
               "status": result["status"], "steps": result["steps"], "sim_time": result["sim_time"],
               "wall_s": result["t_done"] - result["t_submit"], "queue_and_setup_s": result["t_admit"] - result["t_submit"],
               "nu": result["nu"], "ke": result["ke"]}
        return rec

    def write_records(self, path, results):
        """Append the results' records to `path`, one JSON object per line."""
        import json
        with open(path, "a") as f:
            for r in results:
                f.write(json.dumps(self.record(r)) + "\n")

    def cancel(self, rid):
        """Cancel request `rid`; True if it had not finished.  Its result
        (status RBC_ERR_CANCELLED, the steps it advanced) arrives through poll()."""
        found = _I()
        _check(lib().rbc_server_cancel(self._h, int(rid), ctypes.byref(found)))
        return bool(found.value)

    def poll(self, max_results=1024):
        buf = (RbcRequestResult * max_results)()
        n = _I()
        _check(lib().rbc_server_poll(self._h, buf, max_results, ctypes.byref(n)))
        out = []
        for k in range(n.value):
            r = buf[k]
            d = {f: getattr(r, f) for f, _ in RbcRequestResult._fields_}
            # a result is delivered once: its request leaves the table with it
            # (the table holds the requests in flight only)
            d["request"] = self._requests.pop(d["id"], None)
            out.append(d)
        return out

    def wait_idle(self, timeout=60.0):
        idle = _I()
        _check(lib().rbc_server_wait_idle(self._h, float(timeout), ctypes.byref(idle)))
        return bool(idle.value)

    def stats(self):
        st = RbcServerStats()
        _check(lib().rbc_server_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in RbcServerStats._fields_}

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _check(_lib.rbc_server_destroy(h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


MAX_TIMESTEP = 10_000_000


def set_device(ordinal: int):
    """Select the GPU of this thread's library calls (rbc_set_device).  The
    library links its own CUDA runtime, so torch.cuda.set_device does not
    select it."""
    _check(lib().rbc_set_device(int(ordinal)))


def get_device() -> int:
    d = _I()
    _check(lib().rbc_get_device(ctypes.byref(d)))
    return d.value


def set_gemm_wait_limit(polls: int):
    """Test hook: poll limit of the lane GEMM's bounded completion waits on
    the current device (negative: the default).  0 makes every wait time out,
    which exercises the time-out path without a hung GPU."""
    _check(lib().rbc_set_gemm_wait_limit(int(polls)))


def integrate(pde, max_time: float, save_intervall=None, callback=None):
    """integrate() (src/lib.rs:155-187).  ``callback(pde)`` runs at each save
    interval (Integrate::callback); returning True from it stops the loop.
    A Navier2D runs the loop inside the C library (rbc_integrate); any other
    object with the Integrate methods (update, get_time, get_dt, callback,
    exit), e.g. Diffusion2D, runs the same loop here.  Returns the step count."""
    if not isinstance(pde, Navier2D):
        timestep = 0
        dt = pde.get_dt()
        eps_dt = dt * 1e-4
        while True:
            pde.update()
            timestep += 1
            t = pde.get_time()
            if save_intervall:
                r = t % save_intervall
                if r < dt / 2.0 or r > save_intervall - dt / 2.0:
                    out = pde.callback() if callback is None else callback(pde)
                    if callback is not None and out:
                        break
            if t + eps_dt >= max_time or timestep >= MAX_TIMESTEP or pde.exit():
                break
        return timestep
    user_cb = callback if callback is not None else (lambda p: None)

    def _cb(_h, _t, _u):
        return 1 if user_cb(pde) else 0

    cfun = CALLBACK(_cb)
    steps = ctypes.c_long(0)
    _check(lib().rbc_integrate(pde._h, float(max_time), float(save_intervall or 0.0), cfun, None,
                               ctypes.byref(steps)))
    return steps.value


def standard_ic(nav: Navier2D, seed: int = 1, vel_amp: float = 0.2, temp_amp: float = 1e-3):
    """Seeded initial condition of the benchmark configurations: set_velocity(vel_amp, 1, 1),
    interior temperature noise temp_amp*(2u-1) from splitmix64(seed), zero pressure."""
    nav.set_velocity(vel_amp, 1.0, 1.0)
    nav.set_temperature_noise(temp_amp, seed)
    nav.zero_pressure()
