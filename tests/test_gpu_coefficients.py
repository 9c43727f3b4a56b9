"""CoefficientBasedFluxes (coefficient_based_turbulent_fluxes.jl:142-371) on the GPU against
the CPU oracle through the C ABI: constant coefficients, the polynomial neutral drag as the
momentum coefficient, Large-Yeager with FixedIterations(5) and with the default convergence
criteria. Bar as for the similarity-theory solve (tests/test_gpu_ao.py): plain FP64 to 1e-12
relative on 99.99 % of the cells and 1e-11 on every cell, with identical iteration counts; the
FP32 solvers within 1e-5 (errors relative to max(|ref|, 1e-6 max|ref|))."""
import numpy as np
import pytest

from helpers import rel_err, to_numpy
from nesf import api
from nesf import fields as F
from nesf import params as P
from nesf import synthetic as syn
from test_oracle_known_answers import COEFFICIENT_CASES

pytestmark = pytest.mark.gpu

OUT = ("x_momentum", "y_momentum", "sensible_heat", "latent_heat", "water_vapor", "friction_velocity",
       "temperature_scale", "water_vapor_scale")


@pytest.fixture(scope="module")
def state():
    return syn.ao_1deg(nx=180, ny=90)


def run(spec, st, precision):
    import torch
    dev = api.to_device({k: st.fields.get(k) for k in F.AO_INPUTS if k in st.fields})
    out = {k: torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda") for k in F.AO_OUTPUTS}
    it = torch.zeros(st.layout.shape, dtype=torch.int32, device="cuda")
    api.compute_atmosphere_ocean_fluxes(spec, st.layout, dev, out, precision=precision, iterations=it)
    torch.cuda.synchronize()
    res = {k: to_numpy(v) for k, v in out.items()}
    res["iterations"] = to_numpy(it)
    return res


@pytest.mark.parametrize("case", sorted(COEFFICIENT_CASES))
def test_plain_f64_matches_oracle(oracle, state, case):
    spec = P.atmosphere_ocean_interface_spec(flux_formulation=COEFFICIENT_CASES[case]())
    ref = oracle.ao_fluxes(spec.to_c(), state.layout, state.fields)
    gpu = run(spec, state, "f64")
    R = state.layout.ring
    assert np.array_equal(R(gpu["iterations"]), R(ref["iterations"])), case
    for k in OUT:
        e = rel_err(R(gpu[k]), R(ref[k]), floor_frac=1e-6)
        assert np.percentile(e, 99.99) <= 1e-12 and e.max() <= 1e-11, (case, k, float(e.max()))


@pytest.mark.parametrize("precision", ["f32", "f32_adaptive"])
@pytest.mark.parametrize("case", sorted(COEFFICIENT_CASES))
def test_fp32_solvers_within_1e5(oracle, state, case, precision):
    spec = P.atmosphere_ocean_interface_spec(flux_formulation=COEFFICIENT_CASES[case]())
    ref = oracle.ao_fluxes(spec.to_c(), state.layout, state.fields)
    gpu = run(spec, state, precision)
    R = state.layout.ring
    for k in OUT:
        e = rel_err(R(gpu[k]), R(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-5, (case, precision, k, float(e.max()))
