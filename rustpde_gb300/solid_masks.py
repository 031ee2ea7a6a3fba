"""Solid masks for the penalisation term of Navier2D (src/navier/solid_masks.rs).

Each function returns ``[mask, value]`` (physical nx x ny arrays) for
``Navier2D.solid``; the arithmetic runs in the C library
(``rbc_solid_*``), ``solid_porosity_interpolate`` transforms on the GPU.

    nav = Navier2D.new(64, 64, 1e5, 1.0, 0.01, 1.0, adiabatic=True)
    x, y = nav.coords(TEMP)
    nav.solid = solid_cylinder_inner(x, y, 0.2, 0.0, 0.2)
"""
from __future__ import annotations

import numpy as np

from . import _check, _dptr, lib


def _xy(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return x, y, np.empty((x.size, y.size)), np.empty((x.size, y.size))


def solid_cylinder_inner(x, y, x0, y0, radius):
    """Everything with r < radius is solid, with a tanh smoothing layer of
    radius/10 (solid_masks.rs:32-55)."""
    x, y, m, v = _xy(x, y)
    _check(lib().rbc_solid_cylinder_inner(_dptr(x), x.size, _dptr(y), y.size, float(x0), float(y0), float(radius),
                                          _dptr(m), _dptr(v)))
    return [m, v]


def solid_roughness_sinusoid(x, y, height, wavenumber):
    """Sinusoidal roughness elements on both plates (solid_masks.rs:58-98)."""
    x, y, m, v = _xy(x, y)
    _check(lib().rbc_solid_roughness_sinusoid(_dptr(x), x.size, _dptr(y), y.size, float(height), float(wavenumber),
                                              _dptr(m), _dptr(v)))
    return [m, v]


def solid_porosity(x, y, diameter, porosity):
    """A lattice of cylinders mimicking a porous medium (solid_masks.rs:101-140)."""
    x, y, m, v = _xy(x, y)
    _check(lib().rbc_solid_porosity(_dptr(x), x.size, _dptr(y), y.size, float(diameter), float(porosity), _dptr(m),
                                    _dptr(v)))
    return [m, v]


def solid_porosity_interpolate(nx, ny, diameter, porosity):
    """solid_porosity on a 513 x 513 Chebyshev grid, interpolated spectrally
    onto the (nx, ny) Chebyshev grid (solid_masks.rs:144-174).  Needs a GPU."""
    m, v = np.empty((nx, ny)), np.empty((nx, ny))
    _check(lib().rbc_solid_porosity_interpolate(int(nx), int(ny), float(diameter), float(porosity), _dptr(m), _dptr(v)))
    return [m, v]
