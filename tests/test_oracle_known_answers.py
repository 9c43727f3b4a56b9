"""The CPU oracle against the known answers the reference's own tests hold.

test_surface_fluxes.jl:81-110      zero fluxes when dU = dtheta = dq = 0
test_surface_fluxes.jl:148-211     neutral log-law closed form
test_subgrid_velocity_corrections.jl:17-42  ConvectiveGustiness bit identity
test_coefficient_based_fluxes.jl:39-57      linear / Large-Yeager stability values
test_sea_ice_ocean_heat_fluxes.jl:48-178    three-equation interface properties
plus e_sat(T_triple) = p_triple (docs/src/interface_fluxes.md:86-97).
"""
import ctypes as C
import math

import numpy as np
import pytest

from nesf import _abi as A
from nesf import params as P
from nesf import synthetic as syn


def one_cell(**values):
    """A 1x1 exchange grid (halo 2) filled with constant values."""
    L = syn.Layout(1, 1, 2, 2)
    arrs = {k: np.full(L.shape, float(v)) for k, v in values.items()}
    return L, arrs


def test_esat_triple_point(oracle):
    th = P.AtmosphereThermodynamicsParameters().to_c()
    lib = oracle.load()
    for phase in (A.PHASE_LIQUID, A.PHASE_ICE):
        assert lib.oracle_saturation_vapor_pressure(C.byref(th), 273.16, phase) == 611.657


@pytest.mark.parametrize("u,v", [(3.0, -4.0), (0.0, 7.5)])
def test_zero_fluxes(oracle, u, v):
    """dU = 0, dtheta = 0 (lapse-corrected) and q_s = q_a give fluxes below eps(Float32)."""
    spec = P.atmosphere_ocean_interface_spec()
    th = spec.thermodynamics_parameters
    Ta, qa, pa = 15 + 273.15, 0.003, 101325.0
    cp = th.cp_d + (th.water_vapor_heat_capacity - th.cp_d) * qa
    To = Ta - 273.15 + spec.surface_layer_height / cp * spec.gravitational_acceleration
    # the reference mocks q_s = q_a (FixedSpecificHumidity); here the water mole fraction
    # is chosen so that the impure saturation humidity at T_o equals q_a
    einv = 1 / th.Rv_over_Rd
    pv = qa * pa / (einv + (1 - einv) * qa)
    es = syn.esat_liquid(np.float64(To + 273.15), th)
    spec.specific_humidity = P.ImpureSaturationSpecificHumidity("liquid", float(pv / es))
    L, arrs = one_cell(u_atm=u, v_atm=v, T_atm=Ta, p_atm=pa, q_atm=qa, u_oc=u, v_oc=v, T_oc=To, S_oc=35.0)
    out = oracle.ao_fluxes(spec.to_c(), L, arrs)
    eps32 = np.finfo(np.float32).eps
    for k in ("x_momentum", "y_momentum", "sensible_heat", "latent_heat", "water_vapor"):
        assert abs(L.interior(out[k])[0, 0]) < eps32, k


def test_neutral_log_law(oracle):
    """psi = 0, constant roughness 1e-4, no gustiness: u* = k dU / log(h/l) etc."""
    ell = 1e-4
    flux = P.SimilarityTheoryFluxes(momentum_roughness_length=ell, temperature_roughness_length=ell,
                                    water_vapor_roughness_length=ell, subgrid_velocities=None,
                                    stability_functions=None)
    spec = P.atmosphere_ocean_interface_spec(flux_formulation=flux)
    th = spec.thermodynamics_parameters
    ua, va, Ta, qa, pa = 5.5, -2.0, 288.15, 0.003, 100500.0
    L, arrs = one_cell(u_atm=ua, v_atm=va, T_atm=Ta, p_atm=pa, q_atm=qa, u_oc=0, v_oc=0, T_oc=15.0, S_oc=30.0)
    c = spec.to_c()
    out = oracle.ao_fluxes(c, L, arrs)
    lib = oracle.load()
    To = 15.0 + 273.15
    qo = lib.oracle_surface_specific_humidity(C.byref(c), pa, To)
    cp = th.cp_d + (th.water_vapor_heat_capacity - th.cp_d) * qa
    rho = pa / (th.R_d * (1 + (th.Rv_over_Rd - 1) * qa) * Ta)
    Lv = th.reference_vaporization_enthalpy + (th.water_vapor_heat_capacity - th.liquid_water_heat_capacity) * (
        Ta - th.reference_temperature)
    h, g, k = spec.surface_layer_height, spec.gravitational_acceleration, 0.4
    dU = math.hypot(ua, va)
    dth = Ta - To + h / cp * g
    dq = qa - qo
    us = k / math.log(h / ell) * dU
    ts = k / math.log(h / ell) * dth
    qs = k / math.log(h / ell) * dq
    expect = {"x_momentum": -rho * us ** 2 * ua / dU, "y_momentum": -rho * us ** 2 * va / dU,
              "sensible_heat": -rho * cp * us * ts, "water_vapor": -rho * us * qs,
              "latent_heat": -rho * us * qs * Lv}
    for key, val in expect.items():
        assert L.interior(out[key])[0, 0] == pytest.approx(val, rel=1.5e-8), key
    assert L.interior(out["iterations"])[0, 0] == 2     # exact after one step; the second confirms


def test_gustiness_bit_identity(oracle):
    f = P.SimilarityTheoryFluxes().to_c()
    lib = oracle.load()
    for us, bs, hbl in ((0.3, -0.005, 600.0), (0.3, 0.005, 600.0), (1e-4, 0.0, 512.0)):
        Jb = -us * bs
        UG = max(0.01, 1.2 * float(np.cbrt(max(0.0, Jb) * hbl)))
        assert lib.oracle_vsgs2(C.byref(f), us, bs, hbl) == UG ** 2
    assert lib.oracle_vsgs2(C.byref(f), 0.3, -0.005, 600.0) > 0.01 ** 2
    assert lib.oracle_vsgs2(C.byref(f), 0.3, 0.005, 600.0) == 0.01 ** 2
    f0 = P.SimilarityTheoryFluxes(subgrid_velocities=P.ConvectiveGustiness(0, 0)).to_c()
    assert lib.oracle_vsgs2(C.byref(f0), 0.3, -0.005, 600.0) == 0.0
    # SubgridVelocityCorrection composition: convective + mesoscale^2
    vsg = P.mahrt_sun_subgrid_velocity(25e3)
    assert vsg == pytest.approx(0.32 * 4 ** 0.33)
    fs = P.SimilarityTheoryFluxes(subgrid_velocities=P.SubgridVelocityCorrection(P.ConvectiveGustiness(), vsg)).to_c()
    assert lib.oracle_vsgs2(C.byref(fs), 0.3, -0.005, 600.0) == lib.oracle_vsgs2(C.byref(f), 0.3, -0.005, 600.0) + vsg ** 2


def test_stability_values(oracle):
    lib = oracle.load()
    ly = P.large_yeager_stability_functions()
    m, s = ly.momentum.to_c(), ly.temperature.to_c()
    lin = P.SplitStabilityFunction(P.LinearStableStabilityFunction(), P.PaulsonScalarStabilityFunction()).to_c()
    psi = lambda f, z: lib.oracle_stability(C.byref(f), z)
    assert psi(lin, 0.0) == pytest.approx(0.0, abs=1e-12)
    assert psi(lin, 1.0) == pytest.approx(-5.0)
    assert psi(lin, 20.0) == pytest.approx(-50.0)
    assert psi(m, -1.0) > 0
    assert psi(m, 1.0) == pytest.approx(-5.0)
    assert psi(m, 0.0) == pytest.approx(0.0, abs=1e-10)
    assert psi(s, -1.0) > 0
    assert psi(s, 1.0) == pytest.approx(-5.0)


def _edson_momentum_py(z, c):
    zmax, Ap, Bp, Cp, Dp, Am, Bm, Cm, Dm, Em, Fm = c
    zm, zp = min(0.0, z), max(0.0, z)
    dz = min(zmax, Ap * zp)
    psip = -Bp * zp - Cp * (zp - Dp) * math.exp(-dz) - Cp * Dp
    f1 = math.sqrt(math.sqrt(1 - Am * zm))
    psi1 = Bm * math.log((1 + f1) / Bm) + math.log((1 + f1 ** 2) / Bm) - Bm * math.atan(f1) + Cm
    f2 = np.cbrt(1 - Dm * zm)
    psi2 = Em / 2 * math.log((1 + f2 + f2 ** 2) / Em) - math.sqrt(Em) * math.atan((1 + 2 * f2) / math.sqrt(Em)) + Fm
    f = zm ** 2 / (1 + zm ** 2)
    return psip if not z < 0 else (1 - f) * psi1 + f * psi2


def _edson_scalar_py(z, c):
    zmax, Ap, Bp, Cp, Dp, Ep, Am, Bm, Cm, Dm, Em, Fm = c
    zm, zp = min(0.0, z), max(0.0, z)
    dz = min(zmax, Ap * zp)
    psip = -(1 + Bp * zp) ** Cp - Bp * (zp - Dp) * math.exp(-dz) - Ep
    f1 = math.sqrt(1 - Am * zm)
    psi1 = Bm * math.log((1 + f1) / Bm) + Cm
    f2 = np.cbrt(1 - Dm * zm)
    psi2 = Em / 2 * math.log((1 + f2 + f2 ** 2) / Em) - math.sqrt(Em) * math.atan((1 + 2 * f2) / math.sqrt(Em)) + Fm
    f = zm ** 2 / (1 + zm ** 2)
    return psip if not z < 0 else (1 - f) * psi1 + f * psi2


def test_edson_functions_match_independent_restatement(oracle):
    """A second restatement (Python, straight from similarity_theory_turbulent_fluxes.jl:501-618)."""
    lib = oracle.load()
    em, es = P.EdsonMomentumStabilityFunction(), P.EdsonScalarStabilityFunction()
    cm, cs = em.to_c(), es.to_c()
    for z in (-50.0, -3.2, -1.0, -0.1, -1e-6, 0.0, 1e-6, 0.1, 1.0, 7.5, 80.0):
        assert lib.oracle_stability(C.byref(cm), z) == pytest.approx(_edson_momentum_py(z, em.coefficients()), rel=1e-13, abs=1e-15)
        assert lib.oracle_stability(C.byref(cs), z) == pytest.approx(_edson_scalar_py(z, es.coefficients()), rel=1e-13, abs=1e-15)
    # continuity at zero and the neutral limit psi(0) = 0
    assert abs(lib.oracle_stability(C.byref(cm), 0.0)) < 1e-12
    assert abs(lib.oracle_stability(C.byref(cs), -1e-12)) < 1e-9


def _tef(oracle, To, So, Si, us=0.002):
    spec = P.SeaIceOceanSpec(heat_flux=P.ThreeEquationHeatFlux(conductive=False, friction_velocity=us),
                             reference_latent_heat=334e3, ocean_reference_density=1025.0, ocean_heat_capacity=3991.0)
    p = spec.to_c()
    Tb, Sb, q = C.c_double(), C.c_double(), C.c_double()
    oracle.load().oracle_solve_interface_conditions(C.byref(p), To, So, Si, 1.0, 0.1, 0.0,
                                                    C.byref(Tb), C.byref(Sb), C.byref(q))
    return Tb.value, Sb.value, q.value


def test_three_equation_properties(oracle):
    liq = P.LinearLiquidus()
    Tb, Sb, q = _tef(oracle, 2.0, 35.0, 5.0)
    assert 5.0 <= Sb <= 35.0 and Tb == pytest.approx(liq.melting_temperature(Sb)) and q > 0
    Tb, Sb, q = _tef(oracle, liq.melting_temperature(35.0) + 0.5, 35.0, 5.0)
    assert 5.0 <= Sb <= 35.0 and Tb == pytest.approx(liq.melting_temperature(Sb)) and q > 0
    To = liq.melting_temperature(35.0)
    Tb, Sb, q = _tef(oracle, To, 35.0, 5.0)
    assert Sb == pytest.approx(35.0) and Tb == pytest.approx(To) and abs(q) < np.finfo(float).eps
    for So in (30.0, 33.0, 35.0, 37.0, 40.0):
        Tb, Sb, q = _tef(oracle, 1.0, So, 5.0)
        assert 5.0 <= Sb <= So and Tb == pytest.approx(liq.melting_temperature(Sb))
    Tb, Sb, q = _tef(oracle, 1.0, 35.0, 0.0)
    assert 0.0 <= Sb <= 35.0 and Tb == pytest.approx(liq.melting_temperature(Sb))
    for us in (0.1, 0.0001):
        Tb, Sb, q = _tef(oracle, 1.0, 35.0, 5.0, us)
        assert 5.0 <= Sb <= 35.0 and Tb == pytest.approx(liq.melting_temperature(Sb))


def test_ao_solver_converges_on_1deg_sample(oracle):
    """Every cell of a 1-degree sample converges well before maxiter, with physical fluxes."""
    st = syn.ao_1deg(nx=60, ny=30)
    out = oracle.ao_fluxes(P.atmosphere_ocean_interface_spec().to_c(), st.layout, st.fields)
    it = st.layout.ring(out["iterations"])
    assert it.min() >= 2 and it.max() < 100
    us = st.layout.interior(out["friction_velocity"])
    assert np.all(us > 0) and np.all(us < 3)
    assert np.all(np.isfinite(st.layout.interior(out["latent_heat"])))


def test_exact_area_integrals_round_like_fsum():
    """The integral checker's exact sums round to math.fsum of the same FP64 cell terms."""
    import math
    from nesf import synthetic as syn
    from oracle import oracle as O
    rng = np.random.default_rng(8)
    L = syn.Layout(40, 20, 2, 2)
    a = rng.normal(0, 1, L.shape) * 10.0 ** rng.integers(-6, 7, L.shape)
    b = rng.uniform(0, 2, L.shape)
    inactive = (rng.uniform(size=L.shape) < 0.2).astype(np.uint8)
    ex = O.area_integrals(L, [a], [b], inactive=inactive, uniform_area=1.0)[0]
    I = L.interior
    terms = (I(a) * I(b))[I(inactive) == 0]
    assert float(ex) == math.fsum(terms)


# ------------------------------------------------ CoefficientBasedFluxes (§8 f)
def _ly_coefficients():
    return P.CoefficientBasedFluxes(transfer_coefficients=P.LargeYeagerTransferCoefficients()).coefficients_to_c()


def test_polynomial_neutral_drag(oracle):
    """test_coefficient_based_fluxes.jl:16-31: positive and below 5e-3 at 3 m/s, the high-wind
    cap, the wind floor, monotone in moderate winds; and the polynomial at 10 m/s."""
    lib = oracle.load()
    c = _ly_coefficients()
    p = lambda U: lib.oracle_neutral_drag(C.byref(c), U)
    assert 0 < p(3.0) < 5e-3
    assert p(40.0) == pytest.approx(2.34e-3)
    assert p(0.0) == p(0.5)
    assert p(20.0) > p(5.0)
    assert p(10.0) == pytest.approx((2.7 / 10 + 0.142 + 10 / 13.09 - 3.14807e-10 * 1e6) / 1000, rel=1e-14)


def test_large_yeager_defaults():
    """test_coefficient_based_fluxes.jl:59-66, and the library's C defaults equal the Python
    mirror of the reference constructors (LargeYeagerTransferCoefficients, CoefficientBasedFluxes)."""
    from nesf import _lib
    ly = P.LargeYeagerTransferCoefficients()
    assert (ly.reference_height, ly.stable_heat_transfer_coefficient, ly.unstable_heat_transfer_coefficient,
            ly.moisture_transfer_coefficient) == (10.0, 18.0, 32.7, 34.6)
    lib = _lib.load()
    c = A.CoefficientFluxes()
    lib.nesf_default_coefficient_fluxes(C.byref(c), A.COEFFICIENTS_LARGE_YEAGER)
    assert bytes(c) == bytes(_ly_coefficients())
    f = P.CoefficientBasedFluxes()
    assert f.solver_stop_criteria == P.ConvergenceStopCriteria(1e-8, 20)
    with pytest.raises(ValueError):
        P.CoefficientBasedFluxes(transfer_coefficients=(1e-3, 1e-3))
    with pytest.raises(ValueError):
        P.CoefficientBasedFluxes(transfer_coefficients={"momentum": 1e-3})


COEFFICIENT_CASES = {
    # test_coefficient_based_fluxes.jl:90, 123-124, 160-162
    "constant": lambda: P.CoefficientBasedFluxes(transfer_coefficients=(2e-3, 2e-3, 2e-3)),
    "polynomial_drag": lambda: P.CoefficientBasedFluxes(
        transfer_coefficients=(P.PolynomialNeutralDragCoefficient(), 1e-3, 1e-3)),
    "large_yeager_fixed5": lambda: P.CoefficientBasedFluxes(
        transfer_coefficients=P.LargeYeagerTransferCoefficients(), solver_stop_criteria=P.FixedIterations(5)),
    "large_yeager": lambda: P.CoefficientBasedFluxes(transfer_coefficients=P.LargeYeagerTransferCoefficients()),
}


@pytest.mark.parametrize("case", sorted(COEFFICIENT_CASES))
def test_coefficient_based_fluxes_oracle(oracle, case):
    """test_coefficient_based_fluxes.jl:72-178: finite fluxes and u* > 0 with each kind of
    transfer coefficients, on a 1-degree sample; constant coefficients reach their fixed point
    (u* = sqrt(Cd) dU) after two iterations."""
    st = syn.ao_1deg(nx=60, ny=30)
    spec = P.atmosphere_ocean_interface_spec(flux_formulation=COEFFICIENT_CASES[case]())
    out = oracle.ao_fluxes(spec.to_c(), st.layout, st.fields)
    I = st.layout.interior
    for k in ("sensible_heat", "latent_heat", "water_vapor", "x_momentum"):
        assert np.all(np.isfinite(I(out[k]))), k
    assert np.all(I(out["friction_velocity"]) > 0)
    it = st.layout.ring(out["iterations"])
    if case == "constant":
        f = st.fields
        du = I(f["u_atm"]) - (I(f["u_oc"]) + np.roll(I(f["u_oc"]), -1, axis=1)) / 2
        assert np.all(it == 2)
        assert np.all(np.isfinite(du))
    elif case == "large_yeager_fixed5":
        assert np.all(it == 5)
    else:
        assert it.max() <= 20


# ------------------------------------------------ atmosphere-land interface (§8 f)
def _land_cell(T=290.0, Ta=288.0, qa=0.008, u=5.0, sat=1.0):
    L, a = one_cell(u_atm=u, v_atm=0.0, T_atm=Ta, p_atm=101325.0, q_atm=qa, land_temperature=T, saturation=sat)
    return L, a


def _land(oracle, q, **cell):
    L, a = _land_cell(**cell)
    spec = P.atmosphere_land_interface_spec(specific_humidity=q)
    out = oracle.al_fluxes(spec.to_c(), L, a)
    return {k: float(L.interior(v)[0, 0]) for k, v in out.items()}


def test_land_defaults():
    """nesf_default_al_params equals the Python mirror of atmosphere_land_interface's defaults."""
    from nesf import _lib
    lib = _lib.load()
    p = A.InterfaceParams()
    lib.nesf_default_al_params(C.byref(p))
    assert bytes(p) == bytes(P.atmosphere_land_interface_spec().to_c())


def test_bulk_humidity_dry_surface_takes_dew(oracle):
    """interface_states.jl:100-103: a dry surface has q_s = 0, so under humid air the vapor
    flux runs downward (dew/frost); a wet one evaporates into drier air."""
    dry = _land(oracle, P.BulkHumidity(), sat=0.0)
    wet = _land(oracle, P.BulkHumidity(), sat=0.3)
    assert dry["water_vapor"] < 0 and dry["latent_heat"] < 0
    assert wet["water_vapor"] > 0


def test_fractional_humidity_limits(oracle):
    """FractionalHumidity(CriticalSaturation): beta = min(S / S_c, 1); at S >= S_c it is the
    wet BulkHumidity; with a constant beta = 0 the surface is dry."""
    bulk = _land(oracle, P.BulkHumidity(), sat=0.9)
    frac = _land(oracle, P.FractionalHumidity(P.CriticalSaturation(0.75)), sat=0.9)
    for k in ("latent_heat", "sensible_heat", "water_vapor", "friction_velocity"):
        assert frac[k] == bulk[k], k
    dry_b = _land(oracle, P.BulkHumidity(), sat=0.0)
    dry_f = _land(oracle, P.FractionalHumidity(0.0), sat=0.9)
    assert dry_f["water_vapor"] == dry_b["water_vapor"]
    half = _land(oracle, P.FractionalHumidity(P.CriticalSaturation(0.75)), sat=0.375)   # q_s = q_sat / 2
    assert dry_b["water_vapor"] < half["water_vapor"] < bulk["water_vapor"]


def test_skin_humidity_limits(oracle):
    """SkinHumidity (interface_states.jl:600-651): a very conductive soil holds q_s at the
    reservoir's saturation (the wet bulk surface); a sealed soil (kappa_q = 0) drives q_s to
    q_a and the vapor flux to zero."""
    wet = _land(oracle, P.BulkHumidity(), sat=1.0)
    fast = _land(oracle, P.SkinHumidity(surface_thickness=0.01, vapor_diffusivity=1e6))
    assert fast["water_vapor"] == pytest.approx(wet["water_vapor"], rel=1e-6)
    sealed = _land(oracle, P.SkinHumidity(surface_thickness=0.01, vapor_diffusivity=0.0))
    assert abs(sealed["water_vapor"]) < 1e-9 * abs(wet["water_vapor"])
    mid = _land(oracle, P.SkinHumidity())
    assert 0 < mid["water_vapor"] < wet["water_vapor"]


@pytest.mark.parametrize("q", ["bulk", "fractional", "fractional_const", "skin", "dry_layer"])
def test_land_solve_on_1deg_sample(oracle, q):
    """Every model gives finite fluxes and u* > 0 over a 1-degree land sample with dry cells."""
    model = {"bulk": P.BulkHumidity(), "fractional": P.FractionalHumidity(),
             "fractional_const": P.FractionalHumidity(0.5), "skin": P.SkinHumidity(),
             "dry_layer": P.DryLayerHumidity(P.StorageBasedDryLayerDepth(0.05, 0.5),
                                             P.DryLayerVaporPistonVelocity(1e-4, 2.5e-5,
                                                                           tortuosity=P.PowerLawTortuosity()),
                                             thermal_exchange_depth=0.1, porosity=0.4)}[q]
    st = syn.al_1deg(nx=60, ny=30)
    out = oracle.al_fluxes(P.atmosphere_land_interface_spec(specific_humidity=model).to_c(), st.layout, st.fields)
    I = st.layout.interior
    for k in ("latent_heat", "sensible_heat", "water_vapor", "x_momentum"):
        assert np.all(np.isfinite(I(out[k]))), k
    assert np.all(I(out["friction_velocity"]) > 0)
    assert np.array_equal(I(out["interface_temperature"]), I(st.fields["land_temperature"]))


# ------------------------------------------------ DryLayerHumidity (dry_layer_humidity.jl)
# The cases of the reference's test/test_dry_layer_humidity.jl: the humidity function called on
# one state (T_in = 300 K or 310 K against a 290 K bulk land, p = 1e5 Pa, q_a = 0.01,
# T_a = 295 K, u* = 0.3, q* = -2e-4, previous q_s = 0.005), with delta_max = 0.05,
# S_c = 0.5, delta_min = 1e-4, D_0 = 2.5e-5, l_T = 0.1, nu = 0.4.
def _dry_layer_params(exponent=2.0, D0=2.5e-5, width=None, tortuosity=None):
    v = P.DryLayerVaporPistonVelocity(minimum_dry_layer_depth=1e-4, molecular_diffusivity=D0,
                                      wet_transition_width=width, tortuosity=tortuosity or P.ConstantTortuosity())
    q = P.DryLayerHumidity(P.StorageBasedDryLayerDepth(0.05, 0.5, exponent), v, thermal_exchange_depth=0.10,
                           porosity=0.4)
    return P.atmosphere_land_interface_spec(specific_humidity=q).to_c()


def _q_dry(oracle, params, S, Tin=300.0, Tla=290.0, pa=1.0e5, qa=1.0e-2, Ta=295.0, us=0.3, qst=-2.0e-4, qprev=0.005):
    return oracle.load().oracle_dry_layer_humidity(C.byref(params), Tin, Tla, S, Ta, pa, qa, us, qst, qprev)


def _qsat(oracle, params, T, pa=1.0e5):
    return oracle.load().oracle_surface_specific_humidity(C.byref(params), pa, T)


def test_dry_layer_wet_branch(oracle):
    """S = S_c: delta = 0, and with the sharp switch q_s is q_sat(T_in)."""
    p = _dry_layer_params(exponent=2.0, width=0.0)
    assert _q_dry(oracle, p, 0.5) == pytest.approx(_qsat(oracle, p, 300.0), abs=1e-15)


def test_dry_layer_vapor_divider(oracle):
    """S = 0: delta = delta_max, chi = 1/2, and q_s is the conductance-weighted mean of the
    front's q_sat((T_in + T_la) / 2) and q_a."""
    p = _dry_layer_params(exponent=1.0)
    lib = oracle.load()
    qe = _qsat(oracle, p, (300.0 + 290.0) / 2)
    rho = lib.oracle_air_density(C.byref(p.thermo), 295.0, 1.0e5, 1.0e-2)
    Ge = rho * 2.5e-5 / 0.05
    dq = 0.005 - 1.0e-2
    Ja = -rho * 0.3 * -2.0e-4
    Ga = Ja / dq
    expected = (Ge * qe + Ga * 1.0e-2) / (Ge + Ga)
    assert _q_dry(oracle, p, 0.0) == pytest.approx(expected, abs=1e-15)


def test_dry_layer_front_temperature(oracle):
    """A dry layer draws its vapor from a colder front (T_la < T_in): drier than the wet skin."""
    p = _dry_layer_params(exponent=1.0, width=0.0)
    wet = _q_dry(oracle, p, 0.5, Tin=310.0)
    assert wet == pytest.approx(_qsat(oracle, p, 310.0), rel=1e-15)
    assert _q_dry(oracle, p, 0.0, Tin=310.0) < wet


def test_dry_layer_sealed_layer_takes_air_humidity(oracle):
    """G_e -> 0 (D_0 = 1e-14): q_s -> q_a."""
    p = _dry_layer_params(exponent=1.0, D0=1e-14)
    assert _q_dry(oracle, p, 0.0) == pytest.approx(1.0e-2, abs=1e-6)


def test_dry_layer_wet_transition_blend(oracle):
    """The logistic blend: default width 5 delta_min; the sharp switch is exactly wet at S_c;
    the blend stays within 1e-3 of wet there, equals the sharp series solution deep in the dry
    side, and gives the midpoint of wet and series at its centre."""
    assert P.DryLayerVaporPistonVelocity(minimum_dry_layer_depth=1e-4,
                                         molecular_diffusivity=2.5e-5).wet_transition_width == pytest.approx(5e-4)
    sharp = _dry_layer_params(exponent=1.0, width=0.0)
    blend = _dry_layer_params(exponent=1.0, width=1e-2)
    qsat = _qsat(oracle, sharp, 300.0)
    assert _q_dry(oracle, sharp, 0.5) == pytest.approx(qsat, abs=1e-15)
    assert _q_dry(oracle, blend, 0.5) == pytest.approx(qsat, rel=1e-3)
    assert _q_dry(oracle, blend, 0.0) == pytest.approx(_q_dry(oracle, sharp, 0.0), rel=1e-14)
    delta = 1e-4 + 1e-2 / 2
    S_mid = 0.5 * (1 - delta / 0.05)
    assert _q_dry(oracle, blend, S_mid) == pytest.approx((qsat + _q_dry(oracle, sharp, S_mid)) / 2, rel=1e-12)


def test_dry_layer_power_law_tortuosity(oracle):
    """Millington-Quirk (dry_layer_humidity.jl:258-263): at S = 0.2 (eta = 1) the layer is
    delta = 0.03 deep, the front at T_in + 0.3 (T_la - T_in), and D_eff = D_0 theta_g^(10/3) / nu^2
    with theta_g = nu - S nu; q_s is the divider of the two conductances."""
    p = _dry_layer_params(exponent=1.0, tortuosity=P.PowerLawTortuosity())
    lib = oracle.load()
    S, nu = 0.2, 0.4
    delta = 0.05 * (1 - S / 0.5)
    qe = _qsat(oracle, p, 300.0 + min(delta / 0.10, 1.0) * (290.0 - 300.0))
    rho = lib.oracle_air_density(C.byref(p.thermo), 295.0, 1.0e5, 1.0e-2)
    Ge = rho * (2.5e-5 * (nu - S * nu) ** (10 / 3) / nu ** 2) / delta
    Ja = -rho * 0.3 * -2.0e-4
    Ga = Ja / (0.005 - 1.0e-2)
    expected = (Ge * qe + Ga * 1.0e-2) / (Ge + Ga)
    assert _q_dry(oracle, p, S) == pytest.approx(expected, abs=1e-15)
    const = _dry_layer_params(exponent=1.0)
    assert _q_dry(oracle, const, S) != _q_dry(oracle, p, S)


def test_pow_ten_thirds_is_correctly_rounded(oracle):
    """The Millington-Quirk power theta^(10/3) that the oracle (and the kernel, by the same
    construction) takes: the correctly rounded power, checked against 300-bit mpmath."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    f = oracle.load().oracle_pow_ten_thirds
    rng = np.random.default_rng(7)
    xs = np.concatenate([rng.uniform(0, 0.4, 3000), 10 ** rng.uniform(-20, 2, 1000), [1.0, 0.4, 0.125, 1e-300]])
    p = mpmath.mpf(10.0 / 3.0)
    for x in xs:
        assert f(float(x)) == float(mpmath.power(mpmath.mpf(float(x)), p)), float(x)
    assert f(0.0) == 0.0


# ------------------------------------------------ SlabLand flux assembly and land radiation
def _land_assembly(oracle, radiation=None, inactive=None, **values):
    L, a = one_cell(**values)
    if inactive is not None:
        a["inactive"] = np.full(L.shape, inactive, dtype=np.uint8)
    for k in ("surface_energy_flux", "precipitation", "evaporation", "vapor_flux", "liquid_precipitation_flux",
              "upwelling_longwave", "downwelling_longwave", "downwelling_shortwave"):
        a.setdefault(k, np.zeros(L.shape))
    out = oracle.land_assembly(L, a, radiation)
    return {k: float(L.interior(v)[0, 0]) for k, v in out.items()}


def test_slab_land_assembly_cases(oracle):
    """The cases of the reference's test/test_slab_land.jl: evaporation, dew, rain with dew,
    and the turbulent surface energy flux (positive upward)."""
    z = dict(al_sensible=0.0, al_latent=0.0, rain=0.0)
    up = _land_assembly(oracle, **z, al_water_vapor=0.5)
    assert (up["precipitation"], up["evaporation"]) == (0.0, 0.5)
    dew = _land_assembly(oracle, **z, al_water_vapor=-0.5)
    assert (dew["precipitation"], dew["evaporation"]) == (0.5, 0.0)
    wet = _land_assembly(oracle, al_sensible=0.0, al_latent=0.0, al_water_vapor=-0.2, rain=1.5)
    assert wet["precipitation"] == pytest.approx(1.7, abs=1e-12) and wet["evaporation"] == 0.0
    assert wet["liquid_precipitation_flux"] == 1.5 and wet["vapor_flux"] == -0.2
    es = _land_assembly(oracle, al_sensible=2.0, al_latent=-5.0, al_water_vapor=0.0, rain=0.0)
    assert es["surface_energy_flux"] == -3.0


def test_land_radiation_adds_to_surface_energy_flux(oracle):
    """Radiations/apply_air_land_radiative_fluxes.jl as the reference's coupled tests check it:
    the radiation is added to the turbulent surface_energy_flux as -sum_rad, with sum_rad rebuilt
    from the stored diagnostics (downwelling positive into the land, upwelling out); a black
    surface (alpha 0, eps 1) with no incoming radiation raises the flux by sigma T^4."""
    rad = P.LandRadiation(P.SurfaceRadiationProperties(0.2, 0.95)).to_c()
    cell = dict(al_interface_temperature=295.0, sw_down=600.0, lw_down=350.0, surface_energy_flux=-3.0)
    r = _land_assembly(oracle, rad, **cell)
    sum_rad = r["downwelling_longwave"] + r["downwelling_shortwave"] - r["upwelling_longwave"]
    assert r["surface_energy_flux"] == pytest.approx(-3.0 - sum_rad, rel=1e-15)
    assert r["downwelling_shortwave"] == pytest.approx(0.8 * 600.0, rel=1e-15)
    assert r["downwelling_longwave"] == pytest.approx(0.95 * 350.0, rel=1e-15)
    black = P.LandRadiation(P.SurfaceRadiationProperties(0.0, 1.0)).to_c()
    b = _land_assembly(oracle, black, al_interface_temperature=300.0, sw_down=0.0, lw_down=0.0,
                       surface_energy_flux=0.0)
    assert b["upwelling_longwave"] > 0 and b["surface_energy_flux"] == b["upwelling_longwave"]
    assert b["upwelling_longwave"] == pytest.approx(5.670374419e-8 * 300.0 ** 4, rel=1e-15)
    masked = _land_assembly(oracle, rad, **cell, inactive=1)
    assert masked["surface_energy_flux"] == -3.0
