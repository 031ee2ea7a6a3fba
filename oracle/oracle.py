"""Python side of the CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a C++ restatement of rustpde's Rayleigh-Benard time step
(``oracle/rbc_oracle.cpp``).  This module loads it with ctypes and supplies
the one piece the C++ does not restate: the dense real eigen-decomposition
that ``FdmaTensor::from_matrix`` takes from LAPACK geev through
ndarray-linalg (``src/solver/utils.rs:66-98``, ``fdma_tensor.rs:130-141``).
numpy.linalg.eig calls the same LAPACK routine; real parts are kept and the
pairs are sorted by descending eigenvalue, as ``utils::eig`` does.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs may import
this module.  The GPU library never loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle_rbc.so")
_lock = threading.Lock()
_lib = None

# base kinds (rbc_oracle.cpp BaseKind)
CHEB, CD, CN, CDBC, CNBC, FOURIER = 0, 1, 2, 3, 4, 5
# solver kinds
HHOLTZ, HHOLTZ_ADI, POISSON = 0, 1, 2
# Navier2D kinds
BOX_ADIABATIC, BOX_CONDUCTING, PERIODIC = 0, 1, 2
# field ids
TEMP, UX, UY, PRES0, PRES1, FIELDBC, FIELD = 0, 1, 2, 3, 4, 5, 6
# diagnostics
NU, NUVOL, RE, KE, DIVNORM = 0, 1, 2, 3, 4


def build(force: bool = False) -> str:
    """Compile the oracle shared library with make (gcc, OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "rbc_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            P = ctypes.c_void_p
            D = ctypes.c_double
            I = ctypes.c_int
            DP = ctypes.POINTER(ctypes.c_double)
            IP = ctypes.POINTER(ctypes.c_int)
            sig = {
                "or_last_error": (ctypes.c_char_p, []),
                "or_num_threads": (I, []),
                "or_set_threads": (None, [I]),
                "or_set_dense_dct": (None, [I]),
                "or_navier_new": (P, [I, I, D, D, D, D, I]),
                "or_navier_free": (None, [P]),
                "or_navier_tensor_pending": (I, [P, IP]),
                "or_navier_tensor_get": (None, [P, DP, DP]),
                "or_navier_tensor_set": (None, [P, DP, DP, DP]),
                "or_navier_shape": (I, [P, I, IP, IP, IP, IP]),
                "or_navier_get": (None, [P, I, DP]),
                "or_navier_set": (None, [P, I, DP]),
                "or_navier_get_phys": (None, [P, I, DP]),
                "or_navier_coords": (None, [P, I, DP, DP]),
                "or_navier_set_velocity": (None, [P, D, D, D]),
                "or_navier_set_temperature": (None, [P, D, D, D]),
                "or_navier_set_temperature_noise": (None, [P, D, ctypes.c_uint64]),
                "or_navier_zero_pressure": (None, [P]),
                "or_navier_set_solid": (None, [P, DP, DP]),
                "or_navier_update": (I, [P, I]),
                "or_navier_update_many": (I, [ctypes.POINTER(P), I, I]),
                "or_navier_time": (D, [P]),
                "or_navier_set_time": (None, [P, D]),
                "or_navier_eval": (D, [P, I]),
                "or_navier_params": (None, [P, DP]),
                "or_adjoint_new": (P, [I, I, D, D, D, D, I]),
                "or_adjoint_free": (None, [P]),
                "or_adjoint_tensor_pending": (I, [P, I, IP]),
                "or_adjoint_tensor_get": (None, [P, I, DP, DP]),
                "or_adjoint_tensor_set": (None, [P, I, DP, DP, DP]),
                "or_adjoint_shape": (I, [P, I, IP, IP]),
                "or_adjoint_get": (None, [P, I, DP]),
                "or_adjoint_set": (None, [P, I, DP]),
                "or_adjoint_set_velocity": (None, [P, D, D, D]),
                "or_adjoint_set_temperature": (None, [P, D, D, D]),
                "or_adjoint_update": (I, [P, I]),
                "or_adjoint_time": (D, [P]),
                "or_adjoint_eval": (D, [P, I]),
                "or_adjoint_exit": (I, [P]),
                "or_adjoint_residual": (None, [P, DP]),
                "or_lanes_apply": (I, [I, I, I, I, D, DP, DP]),
                "or_space_new": (P, [I, I, I, I]),
                "or_space_free": (None, [P]),
                "or_space_sizes": (I, [P, IP]),
                "or_space_forward": (None, [P, DP, DP]),
                "or_space_backward": (None, [P, DP, DP]),
                "or_space_to_ortho": (None, [P, DP, DP]),
                "or_space_from_ortho": (None, [P, DP, DP]),
                "or_space_gradient": (None, [P, DP, DP, I, I, DP]),
                "or_space_coords": (None, [P, DP, DP, DP, DP]),
                "or_space_average_axis": (None, [P, DP, I, DP]),
                "or_space_average": (D, [P, DP]),
                "or_base_forward": (None, [I, I, DP, DP]),
                "or_base_backward": (None, [I, I, DP, DP]),
                "or_base_to_ortho": (None, [I, I, DP, DP]),
                "or_base_from_ortho": (None, [I, I, DP, DP]),
                "or_base_differentiate": (None, [I, I, DP, DP, I]),
                "or_base_coords": (None, [I, I, DP]),
                "or_base_matrix": (None, [I, I, I, DP, IP, IP]),
                "or_fdma_solve": (None, [DP, I, DP, DP]),
                "or_fdma_solve_c": (None, [DP, I, DP, DP]),
                "or_matvec_fdma": (None, [DP, I, I, DP, I, I, I, DP]),
                "or_solver1d": (None, [I, I, I, D, DP, DP]),
                "or_solver_new": (P, [P, I, D, D]),
                "or_solver_free": (None, [P]),
                "or_solver_tensor_pending": (I, [P, IP]),
                "or_solver_tensor_get": (None, [P, DP, DP]),
                "or_solver_tensor_set": (None, [P, DP, DP, DP]),
                "or_solver_solve": (I, [P, DP, I, I, DP]),
                "or_tensor_new": (P, [DP, DP, I, D]),
                "or_tensor_set": (None, [P, DP, DP, DP]),
                "or_tensor_solve": (None, [P, DP, DP]),
                "or_tensor_free": (None, [P]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a, shape=None, complex_=False) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128 if complex_ else np.float64)
    if shape is not None and a.shape != tuple(shape):
        raise ValueError(f"shape mismatch: got {a.shape}, expected {tuple(shape)}")
    return a


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def num_threads() -> int:
    return lib().or_num_threads()


def set_dense_dct(n: int) -> None:
    """DCT-I of length n by its defining sum instead of the FFT (-1: none):
    an exact restatement of the same transform with other rounding, for
    measuring a case's sensitivity to the transform's rounding."""
    lib().or_set_dense_dct(int(n))


# ---------------------------------------------------------------------------
# eigen-decomposition for FdmaTensor (utils.rs:66-98, fdma_tensor.rs:130-141)
# ---------------------------------------------------------------------------
def tensor_eig(a0: np.ndarray, c0: np.ndarray):
    """Return (lam, fwd, bwd) as FdmaTensor::from_matrix builds them."""
    cinv = np.linalg.inv(c0)
    xmat = cinv @ a0
    lam_c, evec_c = np.linalg.eig(xmat)
    lam = np.ascontiguousarray(lam_c.real)
    evec = np.ascontiguousarray(evec_c.real)
    # argsort ascending (stable, like sort_by), then reversed: largest first
    perm = np.argsort(lam, kind="stable")[::-1]
    lam = np.ascontiguousarray(lam[perm])
    evec = np.ascontiguousarray(evec[:, perm])
    evec_inv = np.linalg.inv(evec)
    fwd = np.ascontiguousarray(evec_inv @ np.linalg.inv(c0))
    return lam, fwd, evec


# ---------------------------------------------------------------------------
# Navier2D
# ---------------------------------------------------------------------------
class Navier2D:
    """Oracle Navier2D (navier.rs).  Use ``Navier2D.new`` / ``new_periodic``."""

    def __init__(self, nx, ny, ra, pr, dt, aspect, kind):
        L = lib()
        self._h = L.or_navier_new(int(nx), int(ny), float(ra), float(pr), float(dt), float(aspect), int(kind))
        if not self._h:
            raise RuntimeError(L.or_last_error().decode())
        self.kind = kind
        self.periodic = kind == PERIODIC
        m = ctypes.c_int(0)
        if L.or_navier_tensor_pending(self._h, ctypes.byref(m)):
            mm = m.value
            a0 = np.zeros((mm, mm))
            c0 = np.zeros((mm, mm))
            L.or_navier_tensor_get(self._h, _dp(a0), _dp(c0))
            lam, fwd, bwd = tensor_eig(a0, c0)
            L.or_navier_tensor_set(self._h, _dp(lam), _dp(fwd), _dp(bwd))
        p = np.zeros(7)
        L.or_navier_params(self._h, _dp(p))
        self.nu, self.ka, self.ra, self.pr, self.dt = p[:5]
        self.scale = p[5:7].copy()

    @classmethod
    def new(cls, nx, ny, ra, pr, dt, aspect, adiabatic=True):
        return cls(nx, ny, ra, pr, dt, aspect, BOX_ADIABATIC if adiabatic else BOX_CONDUCTING)

    @classmethod
    def new_periodic(cls, nx, ny, ra, pr, dt, aspect):
        return cls(nx, ny, ra, pr, dt, aspect, PERIODIC)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_navier_free(h)
            self._h = None

    def shape(self, fid):
        n0, n1, p0, p1 = (ctypes.c_int() for _ in range(4))
        cx = lib().or_navier_shape(self._h, fid, ctypes.byref(n0), ctypes.byref(n1), ctypes.byref(p0), ctypes.byref(p1))
        return (n0.value, n1.value), (p0.value, p1.value), bool(cx)

    def get(self, fid) -> np.ndarray:
        sh, _, cx = self.shape(fid)
        out = np.zeros(sh, dtype=np.complex128 if cx else np.float64)
        lib().or_navier_get(self._h, fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def set(self, fid, arr) -> None:
        sh, _, cx = self.shape(fid)
        a = _f64(arr, sh, cx)
        lib().or_navier_set(self._h, fid, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def get_phys(self, fid) -> np.ndarray:
        _, ph, _ = self.shape(fid)
        out = np.zeros(ph)
        lib().or_navier_get_phys(self._h, fid, _dp(out))
        return out

    def coords(self, fid):
        _, ph, _ = self.shape(fid)
        x = np.zeros(ph[0])
        y = np.zeros(ph[1])
        lib().or_navier_coords(self._h, fid, _dp(x), _dp(y))
        return x, y

    def set_velocity(self, amp, m, n):
        lib().or_navier_set_velocity(self._h, amp, m, n)

    def set_temperature(self, amp, m, n):
        lib().or_navier_set_temperature(self._h, amp, m, n)

    def set_temperature_noise(self, amp, seed):
        lib().or_navier_set_temperature_noise(self._h, amp, ctypes.c_uint64(seed))

    def zero_pressure(self):
        lib().or_navier_zero_pressure(self._h)

    def set_solid(self, mask, value=None):
        """``navier.solid = Some([mask, value])`` (navier.rs:189-190); None clears it."""
        if mask is None:
            lib().or_navier_set_solid(self._h, None, None)
            return
        _, ph, _ = self.shape(TEMP)
        m = np.ascontiguousarray(mask, dtype=np.float64).reshape(ph)
        v = np.zeros(ph) if value is None else np.ascontiguousarray(value, dtype=np.float64).reshape(ph)
        lib().or_navier_set_solid(self._h, _dp(m), _dp(v))

    def update(self, nsteps: int = 1):
        if lib().or_navier_update(self._h, int(nsteps)) != 0:
            raise RuntimeError(lib().or_last_error().decode())

    @property
    def time(self):
        return lib().or_navier_time(self._h)

    @time.setter
    def time(self, t):
        lib().or_navier_set_time(self._h, float(t))

    def eval(self, what):
        return lib().or_navier_eval(self._h, what)

    def exit(self):
        """Integrate::exit for Navier2D (navier.rs:855-862): the L2 norm of the
        divergence is NaN."""
        return bool(np.isnan(self.eval(DIVNORM)))

    def eval_nu(self):
        return self.eval(NU)

    def eval_nuvol(self):
        return self.eval(NUVOL)

    def eval_re(self):
        return self.eval(RE)

    def eval_ke(self):
        return self.eval(KE)

    def div_norm(self):
        return self.eval(DIVNORM)

    def state(self):
        return {f: self.get(f) for f in (TEMP, UX, UY, PRES0, PRES1)}


def update_many(navs, nsteps: int = 1) -> None:
    """Advance independent cases by `nsteps` each, in parallel: one case per
    host thread at a time, in the order given (put the largest first)."""
    arr = (ctypes.c_void_p * len(navs))(*[n._h for n in navs])
    if lib().or_navier_update_many(arr, len(navs), int(nsteps)) != 0:
        raise RuntimeError(lib().or_last_error().decode())


def standard_ic(nav: Navier2D, seed: int = 1, vel_amp: float = 0.2, temp_amp: float = 1e-3):
    """Seeded initial condition shared by the oracle and the GPU path:
    set_velocity(vel_amp, 1, 1) (navier.rs:927), interior temperature noise of
    amplitude temp_amp from splitmix64(seed), zero pressure."""
    nav.set_velocity(vel_amp, 1.0, 1.0)
    nav.set_temperature_noise(temp_amp, seed)
    nav.zero_pressure()


# ---------------------------------------------------------------------------
# funspace primitives
# ---------------------------------------------------------------------------
class Space2:
    def __init__(self, k0, n0, k1, n1):
        self._h = lib().or_space_new(k0, n0, k1, n1)
        s = (ctypes.c_int * 6)()
        self.cpx = bool(lib().or_space_sizes(self._h, s))
        self.phys = (s[0], s[1])
        self.spec = (s[2], s[3])
        self.ortho = (s[4], s[5])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_space_free(h)
            self._h = None

    def _spec_arr(self, shape):
        return np.zeros(shape, dtype=np.complex128 if self.cpx else np.float64)

    def forward(self, v):
        v = _f64(v, self.phys)
        out = self._spec_arr(self.spec)
        lib().or_space_forward(self._h, _dp(v), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def backward(self, vhat):
        vh = _f64(vhat, self.spec, self.cpx)
        out = np.zeros(self.phys)
        lib().or_space_backward(self._h, vh.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _dp(out))
        return out

    def to_ortho(self, vhat):
        vh = _f64(vhat, self.spec, self.cpx)
        out = self._spec_arr(self.ortho)
        lib().or_space_to_ortho(self._h, vh.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def from_ortho(self, o):
        o = _f64(o, self.ortho, self.cpx)
        out = self._spec_arr(self.spec)
        lib().or_space_from_ortho(self._h, o.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def gradient(self, vhat, deriv, scale=None):
        vh = _f64(vhat, self.spec, self.cpx)
        out = self._spec_arr(self.ortho)
        sc = None
        if scale is not None:
            sc_arr = np.asarray(scale, dtype=np.float64)
            sc = _dp(sc_arr)
        lib().or_space_gradient(self._h, vh.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(deriv[0]), int(deriv[1]), sc)
        return out

    def coords(self):
        x0, x1 = np.zeros(self.phys[0]), np.zeros(self.phys[1])
        d0, d1 = np.zeros(self.phys[0]), np.zeros(self.phys[1])
        lib().or_space_coords(self._h, _dp(x0), _dp(x1), _dp(d0), _dp(d1))
        return (x0, x1), (d0, d1)

    def average_axis(self, v, axis):
        v = _f64(v, self.phys)
        out = np.zeros(self.phys[1] if axis == 0 else self.phys[0])
        lib().or_space_average_axis(self._h, _dp(v), int(axis), _dp(out))
        return out

    def average(self, v):
        v = _f64(v, self.phys)
        return lib().or_space_average(self._h, _dp(v))


def lanes_apply(kind, n, op, x, c=0.0):
    """Oracle of the batched 1-D lanes (fs_lanes_apply): op 0 forward, 1
    backward, 2 to_ortho, 3 from_ortho, 4 HholtzAdi solve (coefficient c) on
    every row of x (lanes x length), the rows in parallel."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    m = n - 2 if kind in (CD, CN) else n
    ol = m if op in (0, 3, 4) else n
    out = np.zeros((x.shape[0], ol))
    if lib().or_lanes_apply(int(kind), int(n), int(op), x.shape[0], float(c), _dp(x), _dp(out)) != 0:
        raise RuntimeError(lib().or_last_error().decode())
    return out


class Solver:
    """Hholtz / HholtzAdi / Poisson on a Space2 (2-D)."""

    def __init__(self, space: Space2, kind: int, c):
        self.space = space
        self._h = lib().or_solver_new(space._h, kind, float(c[0]), float(c[1]))
        if not self._h:
            raise RuntimeError(lib().or_last_error().decode())
        m = ctypes.c_int(0)
        if lib().or_solver_tensor_pending(self._h, ctypes.byref(m)):
            mm = m.value
            a0, c0 = np.zeros((mm, mm)), np.zeros((mm, mm))
            lib().or_solver_tensor_get(self._h, _dp(a0), _dp(c0))
            lam, fwd, bwd = tensor_eig(a0, c0)
            lib().or_solver_tensor_set(self._h, _dp(lam), _dp(fwd), _dp(bwd))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_solver_free(h)
            self._h = None

    def solve(self, rhs):
        rhs = _f64(rhs, None, self.space.cpx)
        out = self.space._spec_arr(self.space.spec)
        rc = lib().or_solver_solve(self._h, rhs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), rhs.shape[0], rhs.shape[1],
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        if rc != 0:
            raise RuntimeError(lib().or_last_error().decode())
        return out


def solver1d(basekind, n, kind, c, rhs):
    rhs = _f64(rhs)
    m = n - 2 if basekind in (CD, CN) else n
    out = np.zeros(m)
    lib().or_solver1d(basekind, n, kind, float(c), _dp(rhs), _dp(out))
    return out


def base_forward(kind, n, x):
    x = _f64(x)
    if kind == FOURIER:
        out = np.zeros(n // 2 + 1, dtype=np.complex128)
    else:
        out = np.zeros(n - 2 if kind in (CD, CN) else (2 if kind in (CDBC, CNBC) else n))
    lib().or_base_forward(kind, n, _dp(x), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def base_backward(kind, n, xh):
    xh = _f64(xh, None, kind == FOURIER)
    out = np.zeros(n)
    lib().or_base_backward(kind, n, xh.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _dp(out))
    return out


def base_to_ortho(kind, n, c):
    c = _f64(c)
    out = np.zeros(n)
    lib().or_base_to_ortho(kind, n, _dp(c), _dp(out))
    return out


def base_from_ortho(kind, n, p):
    p = _f64(p)
    out = np.zeros(n - 2 if kind in (CD, CN) else (2 if kind in (CDBC, CNBC) else n))
    lib().or_base_from_ortho(kind, n, _dp(p), _dp(out))
    return out


def base_differentiate(kind, n, c, times):
    if kind == FOURIER:
        c = _f64(c, None, True)
        out = np.zeros(n // 2 + 1, dtype=np.complex128)
    else:
        c = _f64(c)
        out = np.zeros(n)
    lib().or_base_differentiate(kind, n, c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(times))
    return out


def base_coords(kind, n):
    x = np.zeros(n)
    lib().or_base_coords(kind, n, _dp(x))
    return x


def base_matrix(kind, n, which):
    r, c = ctypes.c_int(), ctypes.c_int()
    lib().or_base_matrix(kind, n, which, None, ctypes.byref(r), ctypes.byref(c))
    out = np.zeros((r.value, c.value))
    lib().or_base_matrix(kind, n, which, _dp(out), ctypes.byref(r), ctypes.byref(c))
    return out


def fdma_solve(mat, b):
    mat = _f64(mat)
    n = mat.shape[0]
    if np.iscomplexobj(b):
        b = _f64(b, None, True)
        x = np.zeros(n, dtype=np.complex128)
        lib().or_fdma_solve_c(_dp(mat), n, b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return x
    b = _f64(b)
    x = np.zeros(n)
    lib().or_fdma_solve(_dp(mat), n, _dp(b), _dp(x))
    return x


def matvec_fdma(mat, data, axis):
    mat = _f64(mat)
    data = _f64(data)
    m, n = mat.shape
    shape = (m, data.shape[1]) if axis == 0 else (data.shape[0], m)
    out = np.zeros(shape)
    lib().or_matvec_fdma(_dp(mat), m, n, _dp(data), data.shape[0], data.shape[1], int(axis), _dp(out))
    return out


class Tensor2:
    """FdmaTensor with user-supplied a, c (same pair on both axes)."""

    def __init__(self, a, c, alpha=0.0):
        a = _f64(a)
        c = _f64(c)
        self.n = a.shape[0]
        self._h = lib().or_tensor_new(_dp(a), _dp(c), self.n, float(alpha))
        lam, fwd, bwd = tensor_eig(a, c)
        lib().or_tensor_set(self._h, _dp(lam), _dp(fwd), _dp(bwd))

    def solve(self, b):
        b = _f64(b, (self.n, self.n))
        out = np.zeros((self.n, self.n))
        lib().or_tensor_solve(self._h, _dp(b), _dp(out))
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_tensor_free(h)
            self._h = None


# ---------------------------------------------------------------------------
# Solid masks (src/navier/solid_masks.rs), restated with numpy (elementwise,
# the same arithmetic per grid point as the reference's loops)
# ---------------------------------------------------------------------------
def solid_cylinder_inner(x, y, x0, y0, radius):
    """solid_masks.rs:32-55: mask 1 inside r < radius - radius/10, tanh layer
    0.5 (1 - tanh(2 (r - radius) / layer)) up to radius + radius/10; value 0."""
    x = np.asarray(x, dtype=np.float64)[:, None]
    y = np.asarray(y, dtype=np.float64)[None, :]
    layer = radius / 10.0
    r = np.sqrt((x0 - x) ** 2 + (y0 - y) ** 2)
    smooth = 0.5 * (1.0 - np.tanh(2.0 * (r - radius) / layer))
    mask = np.where(r < radius - layer, 1.0, np.where(r < radius + layer, smooth, 0.0))
    return mask, np.zeros_like(mask)


def solid_roughness_sinusoid(x, y, height, wavenumber):
    """solid_masks.rs:58-98: sinusoidal roughness at both plates, value +0.5
    (bottom) and -0.5 (top); the top assignment wins where both apply."""
    x = np.asarray(x, dtype=np.float64)[:, None]
    y = np.asarray(y, dtype=np.float64)[None, :]
    bottom, top = y[0, 0], y[0, -1]
    layer = height / 10.0
    y_rough = height * (top - bottom) / 2.0 * (np.sin(wavenumber * x) + 0.5)
    shape = (x.shape[0], y.shape[1])
    mask = np.zeros(shape)
    value = np.zeros(shape)
    for y_dist, val in ((y - bottom, 0.5), (top - y, -0.5)):
        y_dist = np.broadcast_to(y_dist, shape)
        yr = np.broadcast_to(y_rough, shape)
        inside = y_dist <= yr
        edge = ~inside & (y_dist <= yr + layer)
        mask = np.where(inside, 1.0, mask)
        mask = np.where(edge, 0.5 * (1.0 - np.tanh(2.0 * (y_dist - yr) / layer)), mask)
        value = np.where(inside | edge, val, value)
    return mask, value


def solid_porosity(x, y, diameter, porosity):
    """solid_masks.rs:101-140: a regular lattice of cylinders whose count per
    axis is round(sqrt((1 - porosity) 4 L^2 / (pi d^2))); masks are summed."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    mask = np.zeros((x.size, y.size))
    radius = diameter / 2.0
    length = x[-1] - x[0]
    height = y[-1] - y[0]
    ncx = np.round(np.sqrt((1.0 - porosity) * 4.0 * length ** 2 / (np.pi * diameter ** 2)))
    ncy = np.round(np.sqrt((1.0 - porosity) * 4.0 * height ** 2 / (np.pi * diameter ** 2)))
    dxs = (length - ncx * diameter) / (ncx + 1.0)
    dys = (height - ncy * diameter) / (ncy + 1.0)
    ox = x[0] + dxs + radius
    for _ in range(int(ncx)):
        oy = y[0] + dys + radius
        for _ in range(int(ncy)):
            mask += solid_cylinder_inner(x, y, ox, oy, radius)[0]
            oy += dys + diameter
        ox += dxs + diameter
    return mask, np.zeros_like(mask)


def solid_porosity_interpolate(nx, ny, diameter, porosity, n_fine=513):
    """solid_masks.rs:144-174: porosity mask on the 513 x 513 Chebyshev grid,
    forward transform, truncation of the coefficients to (nx, ny), backward."""
    fine = Space2(CHEB, n_fine, CHEB, n_fine)
    coarse = Space2(CHEB, nx, CHEB, ny)
    (xf, yf), _ = fine.coords()
    out = []
    for arr in solid_porosity(xf, yf, diameter, porosity):
        vh = fine.forward(arr)
        vc = np.zeros((nx, ny))
        a, b = min(nx, n_fine), min(ny, n_fine)
        vc[:a, :b] = vh[:a, :b]
        out.append(coarse.backward(vc))
    return out[0], out[1]


# ---------------------------------------------------------------------------
# Diffusion2D (src/navier/diffusion.rs:113-238)
# ---------------------------------------------------------------------------
class Diffusion2D:
    """Oracle Diffusion2D: Hholtz solver with c = [dt kappa, dt kappa]
    (diffusion.rs:140-153); update = rhs = to_ortho(vhat), + dt force,
    + dt kappa d2/dx2 fieldbc, + dt kappa d2/dy2 fieldbc, solve
    (diffusion.rs:186-207), in the reference's operation order."""

    def __init__(self, k0, n0, k1, n1, kappa, dt):
        self.space = Space2(k0, n0, k1, n1)
        self.solver = Solver(self.space, HHOLTZ, (dt * kappa, dt * kappa))
        self.kappa, self.dt = kappa, dt
        self.vhat = self.space._spec_arr(self.space.spec)
        self.force = None
        self.bc = None  # (space, vhat, v)
        self.time = 0.0

    def impulse(self):
        """diffusion.rs:156-163"""
        n, m = self.space.phys
        v = np.zeros((n, m))
        v[n // 2, m // 2] = 1.0
        self.vhat = self.space.forward(v)

    def add_force(self, force):
        self.force = np.asarray(force, dtype=np.float64).copy()

    def add_fieldbc(self, k0, k1, vhat):
        sp = Space2(k0, self.space.phys[0], k1, self.space.phys[1])
        self.bc = (sp, np.array(vhat), sp.backward(vhat))

    def update(self, nsteps=1):
        for _ in range(nsteps):
            rhs = self.space.to_ortho(self.vhat)
            if self.force is not None:
                rhs = rhs + self.dt * self.force
            if self.bc is not None:
                sp, bvh, _ = self.bc
                rhs = rhs + self.dt * self.kappa * sp.gradient(bvh, (2, 0), None)
                rhs = rhs + self.dt * self.kappa * sp.gradient(bvh, (0, 2), None)
            self.vhat = self.solver.solve(rhs)
            self.time += self.dt

    def physical(self, with_bc=False):
        v = self.space.backward(self.vhat)
        if with_bc and self.bc is not None:
            v = v + self.bc[2]
        return v



# ---------------------------------------------------------------------------
# Navier2DAdjoint (src/navier/navier_adjoint.rs)
# ---------------------------------------------------------------------------
# adjoint field ids: the state (TEMP, UX, UY, PRES0, PRES1) and the smoothed residuals
TEMP_RES, UX_RES, UY_RES = 10, 11, 12


class Navier2DAdjoint:
    """Oracle Navier2DAdjoint (navier_adjoint.rs): kind as Navier2D."""

    def __init__(self, nx, ny, ra, pr, dt, aspect, kind):
        L = lib()
        self._h = L.or_adjoint_new(int(nx), int(ny), float(ra), float(pr), float(dt), float(aspect), int(kind))
        if not self._h:
            raise RuntimeError(L.or_last_error().decode())
        self.kind = kind
        self.periodic = kind == PERIODIC
        for k in range(5):
            m = ctypes.c_int(0)
            if L.or_adjoint_tensor_pending(self._h, k, ctypes.byref(m)):
                mm = m.value
                a0, c0 = np.zeros((mm, mm)), np.zeros((mm, mm))
                L.or_adjoint_tensor_get(self._h, k, _dp(a0), _dp(c0))
                lam, fwd, bwd = tensor_eig(a0, c0)
                L.or_adjoint_tensor_set(self._h, k, _dp(lam), _dp(fwd), _dp(bwd))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_adjoint_free(h)
            self._h = None

    def get(self, fid):
        n0, n1 = ctypes.c_int(), ctypes.c_int()
        cx = lib().or_adjoint_shape(self._h, fid, ctypes.byref(n0), ctypes.byref(n1))
        out = np.zeros((n0.value, n1.value), dtype=np.complex128 if cx else np.float64)
        lib().or_adjoint_get(self._h, fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def set(self, fid, arr):
        n0, n1 = ctypes.c_int(), ctypes.c_int()
        cx = lib().or_adjoint_shape(self._h, fid, ctypes.byref(n0), ctypes.byref(n1))
        a = _f64(arr, (n0.value, n1.value), bool(cx))
        lib().or_adjoint_set(self._h, fid, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def set_velocity(self, amp, m, n):
        lib().or_adjoint_set_velocity(self._h, amp, m, n)

    def set_temperature(self, amp, m, n):
        lib().or_adjoint_set_temperature(self._h, amp, m, n)

    def update(self, nsteps: int = 1):
        if lib().or_adjoint_update(self._h, int(nsteps)) != 0:
            raise RuntimeError(lib().or_last_error().decode())

    @property
    def time(self):
        return lib().or_adjoint_time(self._h)

    def eval(self, what):
        return lib().or_adjoint_eval(self._h, what)

    def exit(self):
        return bool(lib().or_adjoint_exit(self._h))

    def residual(self):
        """(|u|, |v|, |T|) of the unsmoothed and of the smoothed residual."""
        out = np.zeros(6)
        lib().or_adjoint_residual(self._h, _dp(out))
        return out


MAX_TIMESTEP = 10_000_000


def integrate(pde, dt, max_time, save_intervall=None, callback=None):
    """integrate() (src/lib.rs:155-187) over the oracle: update, the save
    test on time % save_intervall within dt/2 (callback(pde) there), then the
    time limit with eps_dt = dt * 1e-4, MAX_TIMESTEP and exit().  Returns the
    step count."""
    timestep = 0
    eps_dt = dt * 1e-4
    while True:
        pde.update(1)
        timestep += 1
        t = pde.time
        if save_intervall is not None:
            r = t % save_intervall
            if r < dt / 2.0 or r > save_intervall - dt / 2.0:
                if callback is not None:
                    callback(pde)
        if t + eps_dt >= max_time:
            break
        if timestep >= MAX_TIMESTEP:
            break
        if pde.exit():
            break
    return timestep

