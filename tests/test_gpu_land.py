"""The atmosphere-land solve (compute_atmosphere_land_fluxes!, atmosphere_land_fluxes.jl:48-251)
on the GPU against the CPU oracle through the C ABI, for each land humidity model
(BulkHumidity, FractionalHumidity with CriticalSaturation and with a constant efficiency,
SkinHumidity, DryLayerHumidity with either tortuosity and with the sharp wet switch). Bar as
for the ocean: plain FP64 to 1e-12 relative on 99.99 % of the cells and 1e-11 everywhere with
identical iteration counts; the FP32 solvers within 1e-5 (SkinHumidity and DryLayerHumidity
run the FP64 iteration in every mode). Errors are relative to max(|ref|, 1e-6 max|ref|).

SkinHumidity and DryLayerHumidity iterate q_s from a vapor balance, and where the vapor flux
nearly vanishes q_s - q_a cancels: there a one-ulp difference of q_s (from any libm-computed
ingredient: e_sat, the air density, the stability functions) moves the reference's own vapor
fluxes by ulp(q_a) / |q_s - q_a|, up to 1e-10 relative in this sample, and the fixed point
feeds it back with the slope of the q_s map. For those fields the bar is per cell: 4 times the
oracle's response per ulp of q_s (the larger of its responses to a 1024-ulp shift, with and
without the feedback, oracle.humidity_ulp_shift, over 1024: a single ulp rounds away in some
cells), and 1e-12 where that response is smaller. The GPU lands within 2 such units."""
import numpy as np
import pytest

from helpers import rel_err, to_numpy
from nesf import api
from nesf import fields as F
from nesf import params as P
from nesf import synthetic as syn

pytestmark = pytest.mark.gpu


def dry_layer(tortuosity=P.ConstantTortuosity, width=None):
    """DryLayerHumidity with the parameters of the reference's dry-layer tests."""
    return P.DryLayerHumidity(P.StorageBasedDryLayerDepth(0.05, 0.5, 2.0),
                              P.DryLayerVaporPistonVelocity(1e-4, 2.5e-5, wet_transition_width=width,
                                                            tortuosity=tortuosity()),
                              thermal_exchange_depth=0.10, porosity=0.4)


MODELS = {"bulk": P.BulkHumidity, "fractional": P.FractionalHumidity,
          "fractional_const": lambda: P.FractionalHumidity(0.5), "skin": P.SkinHumidity,
          "dry_layer": dry_layer, "dry_layer_power_law": lambda: dry_layer(P.PowerLawTortuosity),
          "dry_layer_sharp": lambda: dry_layer(width=0.0)}
ITERATED_HUMIDITY = ("skin", "dry_layer", "dry_layer_power_law", "dry_layer_sharp")
VAPOR = ("latent_heat", "water_vapor", "water_vapor_scale")
SHIFT_ULPS = 1024
OUT = ("x_momentum", "y_momentum", "sensible_heat", "latent_heat", "water_vapor", "friction_velocity",
       "temperature_scale", "water_vapor_scale", "interface_temperature")


@pytest.fixture(scope="module")
def state():
    return syn.al_1deg(nx=180, ny=90)


def run(spec, st, precision, dtype=None):
    import torch
    dev = api.to_device({k: st.fields[k] for k in F.AL_INPUTS}, dtype=dtype)
    fdt = dev["u_atm"].dtype
    out = {k: torch.zeros(st.layout.shape, dtype=fdt, device="cuda") for k in F.AL_OUTPUTS}
    it = torch.zeros(st.layout.shape, dtype=torch.int32, device="cuda")
    stats = api.compute_atmosphere_land_fluxes(spec, st.layout, dev, out, precision=precision, iterations=it,
                                               stats=True)
    torch.cuda.synchronize()
    res = {k: to_numpy(v).astype(np.float64) for k, v in out.items()}
    res["iterations"] = to_numpy(it)
    return res, stats


@pytest.mark.parametrize("model", sorted(MODELS))
def test_plain_f64_matches_oracle(oracle, state, model):
    spec = P.atmosphere_land_interface_spec(specific_humidity=MODELS[model]())
    ref = oracle.al_fluxes(spec.to_c(), state.layout, state.fields)
    gpu, stats = run(spec, state, "f64")
    I = state.layout.interior
    assert np.array_equal(I(gpu["iterations"]), I(ref["iterations"])), model
    shifted = []
    if model in ITERATED_HUMIDITY:
        for carry in (False, True):
            with oracle.humidity_ulp_shift(SHIFT_ULPS, carry):
                shifted.append(oracle.al_fluxes(spec.to_c(), state.layout, state.fields))
    for k in OUT:
        e = rel_err(I(gpu[k]), I(ref[k]), floor_frac=1e-6)
        if shifted and k in VAPOR:
            s = np.maximum(*(rel_err(I(sh[k]), I(ref[k]), floor_frac=1e-6) for sh in shifted)) / SHIFT_ULPS
            bar = np.maximum(1e-12, 4 * s)
            assert np.all(e <= bar), (model, k, float((e / bar).max()), float(e.max()))
        else:
            assert np.percentile(e, 99.99) <= 1e-12 and e.max() <= 1e-11, (model, k, float(e.max()))
    assert stats["cells"] == state.layout.nx * state.layout.ny


@pytest.mark.parametrize("precision", ["f32", "f32_adaptive"])
@pytest.mark.parametrize("model", sorted(MODELS))
def test_fp32_solvers_within_1e5(oracle, state, model, precision):
    spec = P.atmosphere_land_interface_spec(specific_humidity=MODELS[model]())
    ref = oracle.al_fluxes(spec.to_c(), state.layout, state.fields)
    gpu, stats = run(spec, state, precision)
    I = state.layout.interior
    conv = I(ref["iterations"]) < 100   # where the reference stops at maxiter its answer is its 100th iterate
    for k in OUT:
        e = rel_err(I(gpu[k]), I(ref[k]), floor_frac=1e-6)[conv]
        assert e.max() <= 1e-5, (model, precision, k, float(e.max()))
    if model not in ITERATED_HUMIDITY:
        assert stats["polished"] > 0.5 * stats["cells"]   # the FP32 sweep + FP64 polish ran


def test_fp32_fields(oracle, state):
    """FP32 storage through the FP32 solver: within 1e-5 of the FP64 oracle on the same inputs."""
    spec = P.atmosphere_land_interface_spec()
    f32 = {k: np.asarray(v, dtype=np.float32).astype(np.float64) for k, v in state.fields.items()}
    ref = oracle.al_fluxes(spec.to_c(), state.layout, f32)
    import torch
    gpu, _ = run(spec, state, "f32", dtype=torch.float32)
    I = state.layout.interior
    conv = I(ref["iterations"]) < 100
    for k in OUT:
        e = rel_err(I(gpu[k]), I(ref[k]), floor_frac=1e-6)[conv]
        assert e.max() <= 1e-5, (k, float(e.max()))


def test_land_rejects_ocean_only_options(state):
    from nesf import _lib
    spec = P.atmosphere_land_interface_spec(temperature=P.SkinTemperature(P.DiffusiveFlux()))
    with pytest.raises(_lib.NesfError):
        run(spec, state, "f64")
    spec = P.atmosphere_land_interface_spec(specific_humidity=P.FractionalHumidity(P.CriticalSaturation(0.5)))
    import torch
    dev = api.to_device({k: state.fields[k] for k in F.AL_INPUTS if k != "saturation"})
    out = {k: torch.zeros(state.layout.shape, dtype=torch.float64, device="cuda") for k in F.AL_OUTPUTS}
    with pytest.raises(_lib.NesfError):
        api.compute_atmosphere_land_fluxes(spec, state.layout, dev, out)


def test_dry_layer_rejects_degenerate_parameters(state):
    """Parameters under which the reference divides by zero are refused (NESF_ERR_ARG), and the
    dry-layer model needs the land saturation."""
    from nesf import _lib
    import torch
    for attr in ("minimum_dry_layer_depth", "thermal_exchange_depth"):
        q = dry_layer()
        setattr(q.vapor_exchange if attr == "minimum_dry_layer_depth" else q, attr, 0.0)
        with pytest.raises(_lib.NesfError):
            run(P.atmosphere_land_interface_spec(specific_humidity=q), state, "f64")
    q = dry_layer(P.PowerLawTortuosity)
    q.porosity = 0.0
    with pytest.raises(_lib.NesfError):
        run(P.atmosphere_land_interface_spec(specific_humidity=q), state, "f64")
    dev = api.to_device({k: state.fields[k] for k in F.AL_INPUTS if k != "saturation"})
    out = {k: torch.zeros(state.layout.shape, dtype=torch.float64, device="cuda") for k in F.AL_OUTPUTS}
    with pytest.raises(_lib.NesfError):
        api.compute_atmosphere_land_fluxes(P.atmosphere_land_interface_spec(specific_humidity=dry_layer()),
                                           state.layout, dev, out)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_land_assembly_and_radiation(oracle, state, dtype):
    """nesf_assemble_net_land_fluxes then nesf_apply_air_land_radiative_fluxes against the oracle,
    on the fluxes of the 1-degree land solve with rainfall, radiation and a 10 % mask. FP64 fields:
    identical to the oracle (both built without multiply-add contraction); FP32 fields (FP32
    arithmetic): within 1e-6 of each output's largest magnitude."""
    import torch
    flux = oracle.al_fluxes(P.atmosphere_land_interface_spec().to_c(), state.layout, state.fields)
    rng = np.random.default_rng(5)
    shp = state.layout.shape
    host = {"al_sensible": flux["sensible_heat"], "al_latent": flux["latent_heat"],
            "al_water_vapor": flux["water_vapor"], "al_interface_temperature": flux["interface_temperature"],
            "rain": rng.uniform(0, 1e-4, shp), "sw_down": rng.uniform(0, 1000, shp),
            "lw_down": rng.uniform(250, 450, shp)}
    tdt = torch.float64 if dtype == "f64" else torch.float32
    host = {k: np.asarray(v, dtype=np.float64) if dtype == "f64" else
            np.asarray(v, dtype=np.float32).astype(np.float64) for k, v in host.items()}
    mask = (rng.uniform(size=shp) < 0.1).astype(np.uint8)
    outs = ("surface_energy_flux", "precipitation", "evaporation", "vapor_flux", "liquid_precipitation_flux",
            "upwelling_longwave", "downwelling_longwave", "downwelling_shortwave")
    rad = P.LandRadiation(P.SurfaceRadiationProperties(0.2, 0.95))
    ref = {**{k: v.copy() for k, v in host.items()}, **{k: np.zeros(shp) for k in outs}, "inactive": mask}
    ref = oracle.land_assembly(state.layout, ref)
    ref = oracle.land_assembly(state.layout, ref, rad.to_c())
    dev = {k: torch.tensor(v, dtype=tdt, device="cuda") for k, v in host.items()}
    dev.update({k: torch.zeros(shp, dtype=tdt, device="cuda") for k in outs})
    dev["inactive"] = torch.tensor(mask, device="cuda")
    api.assemble_net_land_fluxes(state.layout, dev)
    api.apply_air_land_radiative_fluxes(rad, state.layout, dev)
    torch.cuda.synchronize()
    I = state.layout.interior
    for k in outs:
        g, r = I(to_numpy(dev[k]).astype(np.float64)), I(ref[k])
        if dtype == "f64":
            assert np.array_equal(g, r), k
        else:
            assert np.abs(g - r).max() <= 1e-6 * np.abs(r).max(), (k, float(np.abs(g - r).max()))


def test_land_assembly_rejects_missing_inputs(state):
    from nesf import _lib
    import torch
    shp = state.layout.shape
    z = lambda: torch.zeros(shp, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.NesfError):
        api.assemble_net_land_fluxes(state.layout, {"al_sensible": z(), "surface_energy_flux": z()})
    with pytest.raises(_lib.NesfError):   # radiation needs T_s, SW, LW and the flux it adds to
        api.apply_air_land_radiative_fluxes(P.LandRadiation(P.SurfaceRadiationProperties(0.2, 0.95)), state.layout,
                                            {"al_interface_temperature": z(), "sw_down": z(), "lw_down": z()})
