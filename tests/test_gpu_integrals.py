"""Compensated FP64 area integrals (nesf_area_integrals) against exact rational sums, and
the ocean heat budget of an assembled coupling step (the reference's conservation check,
test/test_conservation.jl:100-101, 288-291) closed to 1e-12 with FP64 fields."""
from fractions import Fraction

import numpy as np
import pytest

from nesf import api
from nesf import synthetic as syn
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def check_exact(got, exact, scale):
    hi, lo = float(got[0]), float(got[1])
    assert hi == float(exact), (hi, float(exact))
    assert abs(Fraction(hi) + Fraction(lo) - exact) <= Fraction(scale) * Fraction(2) ** -100


def test_integrals_are_exact_with_cancellation_and_mask():
    import torch
    rng = np.random.default_rng(3)
    L = syn.Layout(157, 61, 3, 3)
    # terms spanning 1e-8 .. 1e8 with alternating signs: a plain FP64 sum loses digits
    a = rng.normal(0, 1, L.shape) * 10.0 ** rng.integers(-8, 9, L.shape)
    b = rng.uniform(0.5, 1.5, L.shape)
    area = rng.uniform(1e8, 2e8, L.shape)
    inactive = (rng.uniform(size=L.shape) < 0.3).astype(np.uint8)
    dev = {k: torch.from_numpy(v).cuda() for k, v in dict(a=a, b=b, area=area, inactive=inactive).items()}
    got = api.area_integrals(L, [dev["a"], dev["a"], dev["b"]], [None, dev["b"], None], inactive=dev["inactive"],
                             area=dev["area"]).cpu().numpy()
    exact = O.area_integrals(L, [a, a, b], [None, b, None], inactive=inactive, area=area)
    I = L.interior
    scales = [np.abs(I(a) * I(area)).sum(), np.abs(I(a) * I(b) * I(area)).sum(), np.abs(I(b) * I(area)).sum()]
    for k in range(3):
        check_exact(got[k], exact[k], scales[k])
    again = api.area_integrals(L, [dev["a"], dev["a"], dev["b"]], [None, dev["b"], None], inactive=dev["inactive"],
                               area=dev["area"]).cpu().numpy()
    assert np.array_equal(got, again)   # fixed reduction order


def test_integrals_fp32_fields_row_and_uniform_area():
    import torch
    rng = np.random.default_rng(4)
    L = syn.Layout(300, 40, 2, 2)
    a = rng.normal(0, 300, L.shape).astype(np.float32)
    b = rng.uniform(0, 1, L.shape).astype(np.float32)
    rows = rng.uniform(1e9, 3e9, L.ny)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    got = api.area_integrals(L, [da, da], [None, db], row_area=torch.from_numpy(rows).cuda()).cpu().numpy()
    exact = O.area_integrals(L, [a, a], [None, b], row_area=rows)
    for k in range(2):
        check_exact(got[k], exact[k], np.abs(L.interior(a).astype(np.float64)).sum() * rows.max())
    got = api.area_integrals(L, [da], uniform_area=12345.678).cpu().numpy()
    exact = O.area_integrals(L, [a], uniform_area=12345.678)
    # int dA(a) = sum(a) * A_z: the product of the exact sum and A_z, to ~1e-30
    check_exact(got[0], exact[0], np.abs(L.interior(a).astype(np.float64)).sum() * 12345.678)


def test_ocean_heat_budget_closes():
    from nesf.coupled import CoupledModel
    st = syn.coupled(seed=51, nx=200, ny=100, lat_s=-80, lat_n=80, land=0.3, interpolate=True, dtype=np.float64)
    m = CoupledModel(st)
    m.update_state("f64")
    lhs, rhs, res = m.heat_budget()
    assert abs(lhs) > 0 and res < 1e-12, (lhs, rhs, res)
