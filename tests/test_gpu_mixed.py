"""Mixed-precision step (RBC_PREC_MIXED) against the FP64 oracle.

Dense transforms on the tensor cores (3xTF32, FP32 accumulation), the
convection products in FP32, banded solves / projection / state update in
FP64.  Tolerances: relative L2 per field <= FIELD_TOL after 10 steps; Nusselt
number and kinetic energy <= NU_KE_TOL relative after 100 steps.  A mixed case
inside a batch is bit-identical to the same case stepped alone.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# state fields (temp, ux, uy) and the two pressures: pres[1] is the pressure
# correction potential of the projection, a small difference quantity whose
# relative error is larger than the state's.  The temperature carries the
# error of the transforms (3xTF32, about 1.5e-7 each) on the large linear term
# u.grad(fieldbc).  Largest measured after 10 steps: temp 5.0e-7, ux/uy 9e-9,
# pres[0] 1.1e-7, pres[1] 6.7e-6; the tolerances keep a margin of about 3.
FIELD_TOL = {O.TEMP: 2e-6, O.UX: 1e-7, O.UY: 1e-7, O.PRES0: 5e-7, O.PRES1: 2e-5}
# Nu and KE after 100 steps: 1e-6, the target of the mixed form (largest
# measured: KE of the box 64x64 case at dt = 0.02, 3.3e-7)
NU_KE_TOL = {"box64": 1e-6, "periodic64x33": 1e-6, "periodic512x257": 1e-6}
FIELDS = (O.TEMP, O.UX, O.UY, O.PRES0, O.PRES1)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def R():
    from rustpde_gb300 import build
    build.build()
    import rustpde_gb300
    return rustpde_gb300


CASES = {
    "box64": (O.BOX_ADIABATIC, 64, 64, 1e5, 1.0, 0.02, 1.0),
    "box_cond48x40": (O.BOX_CONDUCTING, 48, 40, 1e6, 0.7, 5e-3, 1.5),
    "periodic64x33": (O.PERIODIC, 64, 33, 1e5, 1.0, 0.005, 1.0),
    "periodic128x64": (O.PERIODIC, 128, 64, 1e6, 0.7, 2e-3, 1.5),
    "periodic512x257": (O.PERIODIC, 512, 257, 1e7, 1.0, 1e-3, 2.0),
    # FP32 mixed-radix Fourier transforms (96 = 2 * 48; odd 45)
    "periodic96x33": (O.PERIODIC, 96, 33, 1e5, 1.0, 0.005, 1.0),
    "periodic45x33": (O.PERIODIC, 45, 33, 1e5, 1.0, 0.005, 1.0),
}


def pair(R, kind, nx, ny, ra, pr, dt, asp, seed=1):
    o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
    O.standard_ic(o, seed)
    g = R.Navier2D(nx, ny, ra, pr, dt, asp, kind, precision=R.PREC_MIXED, seed=None)
    R.standard_ic(g, seed)
    return o, g


@pytest.mark.parametrize("name", list(CASES))
def test_mixed_ten_steps_per_field(R, name):
    o, g = pair(R, *CASES[name])
    o.update(10)
    g.update(10)
    errs = {f: rel(g.get(f), o.get(f)) for f in FIELDS}
    print(name, "relative L2 after 10 steps:", errs)
    for f, e in errs.items():
        assert e < FIELD_TOL[f], (name, f, e)
    assert g.status() == 0


@pytest.mark.parametrize("name", ["box64", "periodic64x33", "periodic512x257"])
def test_mixed_100_steps_nu_ke(R, name):
    o, g = pair(R, *CASES[name])
    o.update(100)
    g.update(100)
    for what in (O.NU, O.KE):
        a, b = g.eval(what), o.eval(what)
        print(name, what, a, b, abs(a - b) / abs(b))
        assert abs(a - b) <= NU_KE_TOL[name] * abs(b), (name, what, a, b)


MIX_PARAMS = [(64, 33, 1e5, 1.0, 0.005, 1.0, O.PERIODIC), (128, 64, 1e6, 0.7, 2e-3, 1.5, O.PERIODIC),
              (64, 33, 1e6, 7.0, 4e-3, 2.0, O.PERIODIC), (48, 40, 1e6, 0.7, 5e-3, 1.5, O.BOX_CONDUCTING),
              (64, 64, 1e5, 1.0, 0.02, 1.0, O.BOX_ADIABATIC)]


# Forms of the FP64 passes (CTA scans, 128-thread CTAs, sub-lane chains) round
# differently in the last bit; in the mixed step a last-bit FP64 difference
# can flip the FP32 rounding of a value fed to the next tensor-core transform,
# so two forms agree to the mixed form's own precision, not to FP64's.
FORMS_TOL = 1e-7


def test_mixed_batch_matches_batch_of_one(R, monkeypatch):
    # batches choose per pass between the forms of the FP64 passes (autotuned
    # on the batch), so a case's numbers match its batch of one up to the
    # roundings of the forms; bitwise identity alone vs in a mix is the
    # serving loop's guarantee (test_gpu_serving.py).  The transforms stay
    # tensor-core GEMMs (";;0"): the butterfly form of a group of 2^p + 1
    # sizes is the FP64 plan, which differs by the mixed form's own error
    monkeypatch.setenv("RBC_BATCH_FORM", ";;0")
    b = R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)
    print("autotuner:", b.tuning())
    for i in range(len(MIX_PARAMS)):
        R.standard_ic(b.cases[i], seed=20 + i)
    b.update(5)
    b.synchronize()
    for i, p in enumerate(MIX_PARAMS):
        one = R.Batch([p], precision=R.PREC_MIXED)
        R.standard_ic(one.cases[0], seed=20 + i)
        one.update(5)
        one.synchronize()
        for f in FIELDS:
            e = rel(b.cases[i].get(f), one.cases[0].get(f))
            assert e < FORMS_TOL, (i, f, e)


def test_mixed_batch_matches_single_case(R, monkeypatch):
    # a single case runs the FP64 passes one CTA per lane (scans): same
    # arithmetic up to the order of the recurrences' roundings (transforms
    # pinned to the GEMMs, as above)
    monkeypatch.setenv("RBC_BATCH_FORM", ";;0")
    b = R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)
    singles = []
    for i, p in enumerate(MIX_PARAMS):
        R.standard_ic(b.cases[i], seed=20 + i)
        s = R.Navier2D(*p, precision=R.PREC_MIXED, seed=None)
        R.standard_ic(s, seed=20 + i)
        singles.append(s)
    b.update(5)
    for s in singles:
        s.update(5)
    b.synchronize()
    for i, s in enumerate(singles):
        for f in FIELDS:
            e = rel(b.cases[i].get(f), s.get(f))
            assert e < FORMS_TOL, (i, f, e)


def test_mixed_batch_forms_replay(R, monkeypatch):
    # the autotuner's forms, replayed through RBC_BATCH_FORM, rebuild the same
    # step: bitwise the same numbers
    b1 = R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)
    forms = b1.tuning_forms()
    assert forms and all(ch in "012345,;" for ch in forms), forms
    monkeypatch.setenv("RBC_BATCH_FORM", forms)
    b2 = R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)
    assert b2.tuning_forms() == forms
    for b in (b1, b2):
        for i in range(len(MIX_PARAMS)):
            R.standard_ic(b.cases[i], seed=40 + i)
        b.update(4)
        b.synchronize()
    for i in range(len(MIX_PARAMS)):
        for f in FIELDS:
            assert np.array_equal(b1.cases[i].get(f), b2.cases[i].get(f)), (i, f)


def test_periodic_y2_fused_form_bitwise(R, monkeypatch):
    # form 3 is form 2 with the periodic Y2 pass's three launches run as one
    # (a CTA barrier between the phases): each thread does the same
    # arithmetic, so the numbers are bitwise the same
    params = MIX_PARAMS + [(45, 33, 1e5, 1.0, 5e-3, 1.0, O.PERIODIC)]
    out = []
    for form in ("2", "3"):
        monkeypatch.setenv("RBC_BATCH_FORM", form)
        b = R.Batch(params, precision=R.PREC_MIXED)
        for i in range(len(params)):
            R.standard_ic(b.cases[i], seed=80 + i)
        b.update(4)
        b.synchronize()
        assert all(b.cases[i].status() == 0 for i in range(len(params)))
        out.append([[b.cases[i].get(f) for f in FIELDS] for i in range(len(params))])
    for i in range(len(params)):
        for k, f in enumerate(FIELDS):
            assert np.array_equal(out[0][i][k], out[1][i][k]), (i, f)


BFLY = [(128, 129, 1e5, 1.0, 5e-3, 1.0, O.PERIODIC), (65, 65, 1e5, 1.0, 1e-2, 1.0, O.BOX_ADIABATIC),
        (129, 129, 1e6, 0.7, 4e-3, 1.5, O.BOX_CONDUCTING), (64, 33, 1e5, 1.0, 5e-3, 1.0, O.PERIODIC)]


def test_transform_gemm_or_butterfly(R, monkeypatch):
    # mixed cases whose Chebyshev lengths are all 2^p + 1 form groups of their
    # own, where the autotuner times the tensor-core GEMM transforms against
    # the butterfly (the group's plain FP64 plan) and keeps the faster: one
    # decision per such group, after the second ';' of the forms
    b = R.Batch(BFLY + [(96, 40, 1e5, 1.0, 5e-3, 1.0, O.PERIODIC)], precision=R.PREC_MIXED)
    parts = b.tuning_forms().split(";")
    assert len(parts) == 3 and len(parts[2].split(",")) == 2, parts  # periodic and box groups
    # pinned to the butterfly, the groups run the FP64 plan: bitwise an FP64 batch
    monkeypatch.setenv("RBC_BATCH_FORM", ";;1")
    bm = R.Batch(BFLY, precision=R.PREC_MIXED)
    assert bm.tuning_forms().split(";")[2] == "1,1"
    bf = R.Batch(BFLY, precision=R.PREC_FP64)
    for bb in (bm, bf):
        for i in range(len(BFLY)):
            R.standard_ic(bb.cases[i], seed=70 + i)
        bb.update(3)
        bb.synchronize()
    for i in range(len(BFLY)):
        assert bm.cases[i].status() == 0
        for f in FIELDS:
            assert np.array_equal(bm.cases[i].get(f), bf.cases[i].get(f)), (i, f)


@pytest.mark.parametrize("gemm_form", ["4", "5"])
def test_wide_gemm_tile_form(R, monkeypatch, gemm_form):
    # GEMM form 4: output tiles of up to 128 columns (one CTA per SM holding all
    # 512 tensor-memory columns) instead of 64; form 5: 64-column tiles in the
    # warp-specialised kernel (producer, MMA and flush warps).  Every other
    # pass as form 0.  The same products, chunk partials and corrections per
    # output element, in the same order: bitwise the same numbers
    params = MIX_PARAMS + [(45, 33, 1e5, 1.0, 5e-3, 1.0, O.PERIODIC)]
    out = []
    for form in ("0", gemm_form):
        monkeypatch.setenv("RBC_BATCH_FORM", "0;" + form)
        b = R.Batch(params, precision=R.PREC_MIXED)
        assert set(b.tuning_forms().replace(",", "").replace(";", "")) <= {form, "0"}
        for i in range(len(params)):
            R.standard_ic(b.cases[i], seed=90 + i)
        b.update(4)
        b.synchronize()
        assert all(b.cases[i].status() == 0 for i in range(len(params)))
        out.append([[b.cases[i].get(f) for f in FIELDS] for i in range(len(params))])
    same = True
    for i in range(len(params)):
        for k, f in enumerate(FIELDS):
            same &= bool(np.array_equal(out[0][i][k], out[1][i][k]))
            assert rel(out[1][i][k], out[0][i][k]) < FORMS_TOL, (i, f)
    assert same


def test_mixed_batch_one_call_equals_single_steps(R, monkeypatch):
    # rbc_batch_step(n) runs the same graph n times as n calls of one step
    # (both batches keep the same forms: the second replays the first's)
    b0 = R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)
    monkeypatch.setenv("RBC_BATCH_FORM", b0.tuning_forms())
    bs = [b0, R.Batch(MIX_PARAMS, precision=R.PREC_MIXED)]
    for b in bs:
        for i in range(len(MIX_PARAMS)):
            R.standard_ic(b.cases[i], seed=60 + i)
    bs[0].update(3)
    for _ in range(3):
        bs[1].update(1)
    for b in bs:
        b.synchronize()
    for i in range(len(MIX_PARAMS)):
        assert bs[0].cases[i].get_time() == bs[1].cases[i].get_time()
        for f in FIELDS:
            assert np.array_equal(bs[0].cases[i].get(f), bs[1].cases[i].get(f)), (i, f)
