"""Seeded synthetic workloads of the batched and serving forms.

``draw_ensemble``: independent RBC cases of uneven size -- (nx, ny) uniform
over {64, 128, 256}^2, box (adiabatic walls) or periodic sidewalls 50/50, Ra
log-uniform in [1e4, 1e8], Pr from {0.7, 1, 7}, aspect uniform in [1, 2],
dt = min(0.02, 2 / sqrt(Ra)).

``draw_requests``: a Poisson arrival stream of solve requests with the same
case distribution plus (512, 257) periodic cases at probability ``p_large``,
and a horizon (simulated time units) uniform in ``horizon``.

All draws use numpy's PCG64 generator with the given seed, so every caller
(bench, tests, serving) sees the same cases.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

BOX_ADIABATIC, BOX_CONDUCTING, PERIODIC = 0, 1, 2
SIZES = (64, 128, 256)
PRANDTL = (0.7, 1.0, 7.0)


def _case(rng):
    nx = int(rng.choice(SIZES))
    ny = int(rng.choice(SIZES))
    kind = PERIODIC if rng.random() < 0.5 else BOX_ADIABATIC
    ra = float(10.0 ** rng.uniform(4.0, 8.0))
    pr = float(rng.choice(PRANDTL))
    aspect = float(rng.uniform(1.0, 2.0))
    dt = min(0.02, 2.0 / math.sqrt(ra))
    return (nx, ny, ra, pr, dt, aspect, kind)


def draw_ensemble(n: int = 256, seed: int = 2024):
    """List of n (nx, ny, ra, pr, dt, aspect, kind) tuples."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return [_case(rng) for _ in range(n)]


@dataclass
class Request:
    rid: int
    arrival: float   # seconds after the stream starts
    params: tuple    # (nx, ny, ra, pr, dt, aspect, kind)
    horizon: float   # simulated time units
    seed: int        # initial-condition seed

    @property
    def steps(self) -> int:
        return max(1, int(round(self.horizon / self.params[4])))

    @property
    def gp(self) -> int:
        return self.params[0] * self.params[1]


def draw_requests(n: int, rate: float = 50.0, seed: int = 7, p_large: float = 0.05, horizon=(1.0, 20.0)):
    """n requests of a Poisson process of `rate` arrivals per second."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        if rng.random() < p_large:
            ra = float(10.0 ** rng.uniform(4.0, 8.0))
            params = (512, 257, ra, float(rng.choice(PRANDTL)), min(0.02, 2.0 / math.sqrt(ra)),
                      float(rng.uniform(1.0, 2.0)), PERIODIC)
        else:
            params = _case(rng)
        h = float(rng.uniform(*horizon))
        out.append(Request(i, t, params, h, 10_000 + i))
    return out
