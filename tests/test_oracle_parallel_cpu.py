"""The oracle's case-parallel update (the CPU ensemble sample) advances every
case exactly as its own sequential update does: bit-identical fields, the
same time (no GPU is used)."""
import numpy as np

from oracle import oracle as O


def test_update_many_equals_sequential():
    params = [(32, 33, 1e5, 1.0, 0.01, 1.0, O.BOX_ADIABATIC), (48, 33, 1e5, 0.7, 0.005, 2.0, O.PERIODIC),
              (33, 33, 3e4, 1.0, 0.01, 1.0, O.BOX_CONDUCTING), (64, 17, 1e5, 1.0, 0.005, 1.0, O.PERIODIC),
              (16, 16, 1e5, 1.0, 0.02, 1.0, O.BOX_ADIABATIC)]
    seq, par = [], []
    for i, p in enumerate(params):
        for lst in (seq, par):
            o = O.Navier2D(*p)
            O.standard_ic(o, 40 + i)
            lst.append(o)
    for o in seq:
        o.update(3)
    O.set_threads(4)
    O.update_many(par, 3)
    for a, b in zip(seq, par):
        assert a.time == b.time
        for f in (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1):
            assert np.array_equal(a.get(f), b.get(f)), f
