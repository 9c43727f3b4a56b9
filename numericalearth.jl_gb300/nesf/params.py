"""Host-side mirror of NumericalEarth.jl's interface-flux parameter types.

Each class keeps the reference's name, keyword names and defaults, and knows how
to pack itself into the POD structs of include/nesf.h. Citations are paths inside
NumericalEarth.jl v0.6.2.
"""
import math
from dataclasses import dataclass, field
from typing import Optional, Union

from . import _abi as A

# Oceananigans.defaults.gravitational_acceleration (EarthSystemModels.jl:70)
default_gravitational_acceleration = 9.80665
celsius_to_kelvin = 273.15          # components.jl:10
default_stefan_boltzmann_constant = 5.670374419e-8   # Radiations.jl:13
default_water_emissivity = 0.97     # Radiations.jl:16


# ---------------------------------------------------------------- thermodynamics
@dataclass
class AtmosphereThermodynamicsParameters:
    """src/Atmospheres/thermodynamic_parameters.jl:61-69,106-116,149-165,220-226."""
    gas_constant: float = 8.3144598
    dry_air_molar_mass: float = 0.02897
    water_molar_mass: float = 0.018015
    dry_air_adiabatic_exponent: float = 2 / 7
    water_vapor_heat_capacity: float = 1859.0
    liquid_water_heat_capacity: float = 4181.0
    water_ice_heat_capacity: float = 2100.0
    reference_vaporization_enthalpy: float = 2500800.0
    reference_sublimation_enthalpy: float = 2834400.0
    reference_temperature: float = 273.16
    triple_point_temperature: float = 273.16
    triple_point_pressure: float = 611.657

    def to_c(self):
        return A.ThermodynamicsParameters(*[getattr(self, n) for n, _ in A.ThermodynamicsParameters._fields_])

    # Derived quantities (thermodynamic_parameters.jl:73-78, 256)
    @property
    def R_d(self):
        return self.gas_constant / self.dry_air_molar_mass

    @property
    def R_v(self):
        return self.gas_constant / self.water_molar_mass

    @property
    def Rv_over_Rd(self):
        return self.dry_air_molar_mass / self.water_molar_mass

    @property
    def cp_d(self):
        return self.R_d / self.dry_air_adiabatic_exponent


# --------------------------------------------------------------- stability functions
class AbstractStabilityFunction:
    kind = A.PSI_ZERO

    def coefficients(self):
        return []

    def to_c(self):
        s = A.StabilityFunction()
        s.kind = self.kind
        for n, v in enumerate(self.coefficients()):
            s.c[n] = v
        return s


class ZeroStabilityFunction(AbstractStabilityFunction):
    """psi == 0 (the `zero_stability_function` of test_surface_fluxes.jl:155)."""
    kind = A.PSI_ZERO


@dataclass
class EdsonMomentumStabilityFunction(AbstractStabilityFunction):
    """similarity_theory_turbulent_fluxes.jl:487-499."""
    ζmax: float = 50.0
    A_plus: float = 0.35
    B_plus: float = 0.7
    C_plus: float = 0.75
    D_plus: float = 5 / 0.35
    A_minus: float = 15.0
    B_minus: float = 2.0
    C_minus: float = math.pi / 2
    D_minus: float = 10.15
    E_minus: float = 3.0
    F_minus: float = math.pi / math.sqrt(3)
    kind = A.PSI_EDSON_MOMENTUM

    def coefficients(self):
        return [self.ζmax, self.A_plus, self.B_plus, self.C_plus, self.D_plus, self.A_minus,
                self.B_minus, self.C_minus, self.D_minus, self.E_minus, self.F_minus]


@dataclass
class EdsonScalarStabilityFunction(AbstractStabilityFunction):
    """similarity_theory_turbulent_fluxes.jl:571-584."""
    ζmax: float = 50.0
    A_plus: float = 0.35
    B_plus: float = 2 / 3
    C_plus: float = 3 / 2
    D_plus: float = 14.28
    E_plus: float = 8.525
    A_minus: float = 15.0
    B_minus: float = 2.0
    C_minus: float = 0.0
    D_minus: float = 34.15
    E_minus: float = 3.0
    F_minus: float = math.pi / math.sqrt(3)
    kind = A.PSI_EDSON_SCALAR

    def coefficients(self):
        return [self.ζmax, self.A_plus, self.B_plus, self.C_plus, self.D_plus, self.E_plus,
                self.A_minus, self.B_minus, self.C_minus, self.D_minus, self.E_minus, self.F_minus]


@dataclass
class ShebaMomentumStabilityFunction:
    """similarity_theory_turbulent_fluxes.jl:637-640."""
    a: float = 6.5
    b: float = 1.3


@dataclass
class ShebaScalarStabilityFunction:
    """similarity_theory_turbulent_fluxes.jl:659-663."""
    a: float = 5.0
    b: float = 5.0
    c: float = 3.0


@dataclass
class PaulsonMomentumStabilityFunction:
    """similarity_theory_turbulent_fluxes.jl:683-686."""
    a: float = 16.0
    b: float = math.pi / 2


@dataclass
class PaulsonScalarStabilityFunction:
    """similarity_theory_turbulent_fluxes.jl:701-703."""
    a: float = 16.0


@dataclass
class LinearStableStabilityFunction:
    """similarity_theory_turbulent_fluxes.jl:742-745."""
    coefficient: float = 5.0
    maximum_stability_parameter: float = 10.0


@dataclass
class SplitStabilityFunction(AbstractStabilityFunction):
    """similarity_theory_turbulent_fluxes.jl:712-725: stable branch for zeta > 0."""
    stable: object = None
    unstable: object = None

    @property
    def kind(self):
        st, un = type(self.stable), type(self.unstable)
        if st is ShebaMomentumStabilityFunction and un is PaulsonMomentumStabilityFunction:
            return A.PSI_SHEBA_PAULSON_MOMENTUM
        if st is ShebaScalarStabilityFunction and un is PaulsonScalarStabilityFunction:
            return A.PSI_SHEBA_PAULSON_SCALAR
        if st is LinearStableStabilityFunction and un is PaulsonMomentumStabilityFunction:
            return A.PSI_LINEAR_PAULSON_MOMENTUM
        if st is LinearStableStabilityFunction and un is PaulsonScalarStabilityFunction:
            return A.PSI_LINEAR_PAULSON_SCALAR
        raise NotImplementedError(f"SplitStabilityFunction({st.__name__}, {un.__name__})")

    def coefficients(self):
        k = self.kind
        s, u = self.stable, self.unstable
        if k == A.PSI_SHEBA_PAULSON_MOMENTUM:
            return [s.a, s.b, u.a, u.b]
        if k == A.PSI_SHEBA_PAULSON_SCALAR:
            return [s.a, s.b, s.c, u.a]
        if k == A.PSI_LINEAR_PAULSON_MOMENTUM:
            return [s.coefficient, s.maximum_stability_parameter, u.a, u.b]
        return [s.coefficient, s.maximum_stability_parameter, u.a]


@dataclass
class SimilarityScales:
    """similarity_theory_turbulent_fluxes.jl:432-436."""
    momentum: object
    temperature: object
    water_vapor: object


def atmosphere_ocean_stability_functions():
    """similarity_theory_turbulent_fluxes.jl:621-625 (Edson et al. 2013)."""
    psc = EdsonScalarStabilityFunction()
    return SimilarityScales(EdsonMomentumStabilityFunction(), psc, psc)


def atmosphere_sea_ice_stability_functions():
    """similarity_theory_turbulent_fluxes.jl:779-789 (Paulson unstable, SHEBA stable)."""
    m = SplitStabilityFunction(ShebaMomentumStabilityFunction(), PaulsonMomentumStabilityFunction())
    s = SplitStabilityFunction(ShebaScalarStabilityFunction(), PaulsonScalarStabilityFunction())
    return SimilarityScales(m, s, s)


def large_yeager_stability_functions():
    """similarity_theory_turbulent_fluxes.jl:766-771."""
    st = LinearStableStabilityFunction()
    return SimilarityScales(SplitStabilityFunction(st, PaulsonMomentumStabilityFunction()),
                            SplitStabilityFunction(st, PaulsonScalarStabilityFunction()),
                            SplitStabilityFunction(st, PaulsonScalarStabilityFunction()))


# ----------------------------------------------------------------- roughness lengths
@dataclass
class WindDependentWaveFormulation:
    """roughness_lengths.jl:56-75."""
    Umax: float = 19.0
    C1: float = 0.0017
    C2: float = -0.005


@dataclass
class TemperatureDependentAirViscosity:
    """roughness_lengths.jl:149-189."""
    C0: float = 1.326e-5
    C1: float = 1.326e-5 * 6.542e-3
    C2: float = 1.326e-5 * 8.301e-6
    C3: float = -1.326e-5 * 4.84e-9


@dataclass
class ReynoldsScalingFunction:
    """roughness_lengths.jl:212-231."""
    A: float = 5.85e-5
    b: float = 0.72


def _viscosity_into(c, nu):
    if isinstance(nu, TemperatureDependentAirViscosity):
        c.viscosity_kind = 1
        for n, v in enumerate((nu.C0, nu.C1, nu.C2, nu.C3)):
            c.viscosity_coefficients[n] = v
    else:
        c.viscosity_kind = 0
        c.air_kinematic_viscosity = float(nu)


@dataclass
class MomentumRoughnessLength:
    """roughness_lengths.jl:123-139."""
    gravitational_acceleration: float = default_gravitational_acceleration
    maximum_roughness_length: float = 1.0
    air_kinematic_viscosity: Union[float, TemperatureDependentAirViscosity] = 1.5e-5
    wave_formulation: Union[float, WindDependentWaveFormulation] = 0.02
    smooth_wall_parameter: float = 0.11

    def to_c(self):
        c = A.RoughnessLength()
        c.kind = A.ROUGHNESS_MOMENTUM
        c.gravitational_acceleration = self.gravitational_acceleration
        _viscosity_into(c, self.air_kinematic_viscosity)
        if isinstance(self.wave_formulation, WindDependentWaveFormulation):
            c.wave_kind = 1
            c.wave_umax = self.wave_formulation.Umax
            c.wave_c1 = self.wave_formulation.C1
            c.wave_c2 = self.wave_formulation.C2
        else:
            c.wave_kind = 0
            c.charnock = float(self.wave_formulation)
        c.smooth_wall_parameter = self.smooth_wall_parameter
        c.maximum_roughness_length = self.maximum_roughness_length
        return c


@dataclass
class ScalarRoughnessLength:
    """roughness_lengths.jl:93-101."""
    air_kinematic_viscosity: Union[float, TemperatureDependentAirViscosity] = 1.5e-5
    reynolds_number_scaling_function: ReynoldsScalingFunction = field(default_factory=ReynoldsScalingFunction)
    maximum_roughness_length: float = 1.6e-4

    def to_c(self):
        c = A.RoughnessLength()
        c.kind = A.ROUGHNESS_SCALAR
        _viscosity_into(c, self.air_kinematic_viscosity)
        c.reynolds_A = self.reynolds_number_scaling_function.A
        c.reynolds_b = self.reynolds_number_scaling_function.b
        c.maximum_roughness_length = self.maximum_roughness_length
        return c


def _roughness_to_c(r):
    if isinstance(r, (int, float)):
        c = A.RoughnessLength()
        c.kind = A.ROUGHNESS_CONSTANT
        c.value = float(r)
        return c
    return r.to_c()


# ------------------------------------------------------------ subgrid velocities
@dataclass
class ConvectiveGustiness:
    """similarity_theory_turbulent_fluxes.jl:45-48."""
    gustiness_parameter: float = 1.2
    minimum_gustiness: float = 0.01


@dataclass
class SubgridVelocityCorrection:
    """similarity_theory_turbulent_fluxes.jl:69-80 (convective slot + static mesoscale slot)."""
    convective: object = field(default_factory=ConvectiveGustiness)
    mesoscale: Optional[float] = None


def mahrt_sun_subgrid_velocity(dx, threshold=5e3):
    """similarity_theory_turbulent_fluxes.jl:114-117."""
    delta = max(dx / threshold - 1, 0)
    return 0.32 * delta ** 0.33


# ---------------------------------------------------------------- stop criteria
@dataclass
class ConvergenceStopCriteria:
    """compute_interface_state.jl:5-8."""
    tolerance: float = 1e-8
    maxiter: int = 100


@dataclass
class FixedIterations:
    """compute_interface_state.jl:20-22."""
    iterations: int = 10


# --------------------------------------------------------- SimilarityTheoryFluxes
@dataclass
class SimilarityTheoryFluxes:
    """similarity_theory_turbulent_fluxes.jl:174-214 (keyword names and defaults)."""
    von_karman_constant: float = 0.4
    turbulent_prandtl_number: float = 1.0
    subgrid_velocities: object = field(default_factory=ConvectiveGustiness)
    stability_functions: Optional[SimilarityScales] = field(default_factory=atmosphere_ocean_stability_functions)
    momentum_roughness_length: object = field(default_factory=MomentumRoughnessLength)
    temperature_roughness_length: object = field(default_factory=ScalarRoughnessLength)
    water_vapor_roughness_length: object = field(default_factory=ScalarRoughnessLength)
    zero_plane_displacement: float = 0.0
    similarity_form: str = "logarithmic"
    solver_stop_criteria: object = None
    solver_tolerance: float = 1e-8
    solver_maxiter: int = 100

    def __post_init__(self):
        if self.solver_stop_criteria is None:
            self.solver_stop_criteria = ConvergenceStopCriteria(self.solver_tolerance, self.solver_maxiter)
        if self.stability_functions is None:
            z = ZeroStabilityFunction()
            self.stability_functions = SimilarityScales(z, z, z)

    def to_c(self):
        c = A.SimilarityTheoryFluxesC()
        c.von_karman_constant = self.von_karman_constant
        c.turbulent_prandtl_number = self.turbulent_prandtl_number
        sv = self.subgrid_velocities
        meso = None
        if isinstance(sv, SubgridVelocityCorrection):
            meso = sv.mesoscale
            sv = sv.convective
        if sv is None:
            c.subgrid_kind = A.SUBGRID_NONE
        elif isinstance(sv, (int, float)):
            c.subgrid_kind = A.SUBGRID_CONSTANT
            c.constant_subgrid_velocity = float(sv)
        else:
            c.subgrid_kind = A.SUBGRID_CONVECTIVE
            c.gustiness_parameter = sv.gustiness_parameter
            c.minimum_gustiness = sv.minimum_gustiness
        c.mesoscale_subgrid_velocity = 0.0 if meso is None else float(meso)
        c.similarity_form = A.PROFILE_COARE if self.similarity_form == "coare" else A.PROFILE_LOGARITHMIC
        sf = self.stability_functions
        for n, psi in enumerate((sf.momentum, sf.temperature, sf.water_vapor)):
            c.stability[n] = psi.to_c()
        for n, r in enumerate((self.momentum_roughness_length, self.temperature_roughness_length,
                               self.water_vapor_roughness_length)):
            c.roughness[n] = _roughness_to_c(r)
        c.zero_plane_displacement = self.zero_plane_displacement
        sc = self.solver_stop_criteria
        if isinstance(sc, FixedIterations):
            c.stop_kind = A.STOP_FIXED_ITERATIONS
            c.maxiter = sc.iterations
            c.tolerance = 0.0
        else:
            c.stop_kind = A.STOP_CONVERGENCE
            c.maxiter = sc.maxiter
            c.tolerance = sc.tolerance
        return c


# ------------------------------------------------------- CoefficientBasedFluxes
@dataclass
class PolynomialNeutralDragCoefficient:
    """coefficient_based_turbulent_fluxes.jl:20-54 (Large & Yeager 2004)."""
    a: float = 2.7
    b: float = 0.142
    c: float = 1 / 13.09
    d: float = 3.14807e-10
    high_wind_speed_threshold: float = 33.0
    high_wind_drag_coefficient: float = 2.34e-3
    minimum_wind_speed: float = 0.5


@dataclass
class LargeYeagerTransferCoefficients:
    """coefficient_based_turbulent_fluxes.jl:82-108."""
    von_karman_constant: float = 0.4
    neutral_drag_coefficient: PolynomialNeutralDragCoefficient = field(
        default_factory=PolynomialNeutralDragCoefficient)
    stability_functions: SimilarityScales = field(default_factory=large_yeager_stability_functions)
    reference_height: float = 10.0
    stable_heat_transfer_coefficient: float = 18.0
    unstable_heat_transfer_coefficient: float = 32.7
    moisture_transfer_coefficient: float = 34.6


@dataclass
class CoefficientBasedFluxes:
    """coefficient_based_turbulent_fluxes.jl:142-258 (keyword names and defaults):
    transfer_coefficients a 3-tuple / dict of constants (momentum, temperature,
    water_vapor) or LargeYeagerTransferCoefficients."""
    transfer_coefficients: object = (1e-3, 1e-3, 1e-3)
    solver_stop_criteria: object = None
    solver_tolerance: float = 1e-8
    solver_maxiter: int = 20

    def __post_init__(self):
        if self.solver_stop_criteria is None:
            self.solver_stop_criteria = ConvergenceStopCriteria(self.solver_tolerance, self.solver_maxiter)
        tc = self.transfer_coefficients
        if isinstance(tc, dict):
            missing = [k for k in ("momentum", "temperature", "water_vapor") if k not in tc]
            if missing:
                raise ValueError(f"transfer coefficients must contain momentum, temperature, water_vapor; "
                                 f"missing {missing}")
        elif not isinstance(tc, LargeYeagerTransferCoefficients) and len(tc) != 3:
            raise ValueError(f"transfer coefficients must be (momentum, temperature, water_vapor), got {tc}")

    def coefficients_to_c(self):
        c = A.CoefficientFluxes()
        sc = self.solver_stop_criteria
        if isinstance(sc, FixedIterations):
            c.stop_kind, c.maxiter, c.tolerance = A.STOP_FIXED_ITERATIONS, sc.iterations, 0.0
        else:
            c.stop_kind, c.maxiter, c.tolerance = A.STOP_CONVERGENCE, sc.maxiter, sc.tolerance
        tc = self.transfer_coefficients
        if isinstance(tc, LargeYeagerTransferCoefficients):
            c.kind = A.COEFFICIENTS_LARGE_YEAGER
            n = tc.neutral_drag_coefficient
            c.von_karman_constant = tc.von_karman_constant
            c.drag_a, c.drag_b, c.drag_c, c.drag_d = n.a, n.b, n.c, n.d
            c.high_wind_speed_threshold = n.high_wind_speed_threshold
            c.high_wind_drag_coefficient = n.high_wind_drag_coefficient
            c.minimum_wind_speed = n.minimum_wind_speed
            c.reference_height = tc.reference_height
            c.stable_heat_transfer_coefficient = tc.stable_heat_transfer_coefficient
            c.unstable_heat_transfer_coefficient = tc.unstable_heat_transfer_coefficient
            c.moisture_transfer_coefficient = tc.moisture_transfer_coefficient
            c.stability[0] = tc.stability_functions.momentum.to_c()
            c.stability[1] = tc.stability_functions.temperature.to_c()
        else:
            c.kind = A.COEFFICIENTS_CONSTANT
            vals = (tc["momentum"], tc["temperature"], tc["water_vapor"]) if isinstance(tc, dict) else tuple(tc)
            poly = [v for v in vals if isinstance(v, PolynomialNeutralDragCoefficient)]
            if any(p != poly[0] for p in poly):
                raise NotImplementedError("one PolynomialNeutralDragCoefficient per CoefficientBasedFluxes")
            if poly:   # evaluate_coefficient(C::PolynomialNeutralDragCoefficient, dU) = C(dU)
                n = poly[0]
                c.drag_a, c.drag_b, c.drag_c, c.drag_d = n.a, n.b, n.c, n.d
                c.high_wind_speed_threshold = n.high_wind_speed_threshold
                c.high_wind_drag_coefficient = n.high_wind_drag_coefficient
                c.minimum_wind_speed = n.minimum_wind_speed
            mask = 0
            for i, v in enumerate(vals):
                if isinstance(v, PolynomialNeutralDragCoefficient):
                    mask |= 1 << i
                    v = 0.0
                setattr(c, ("momentum", "temperature", "water_vapor")[i], float(v))
            c.polynomial_mask = mask
        return c


def atmosphere_sea_ice_similarity_theory(**kw):
    """similarity_theory_turbulent_fluxes.jl:791-794."""
    return SimilarityTheoryFluxes(stability_functions=atmosphere_sea_ice_stability_functions(), **kw)


# ----------------------------------------------------------- interface formulations
@dataclass
class ImpureSaturationSpecificHumidity:
    """interface_states.jl:20-24,44 (phase "liquid" | "ice"; water_mole_fraction None = 1)."""
    phase: str = "liquid"
    water_mole_fraction: Optional[float] = None


@dataclass
class BulkHumidity:
    """interface_states.jl:100-125: q_sat(T_s) where the land saturation > 0, else 0."""
    phase: str = "liquid"


@dataclass
class CriticalSaturation:
    """interface_states.jl:128-158: beta = min(S / S_c, 1) (Manabe 1969)."""
    critical_saturation: float = 0.75


@dataclass
class FractionalHumidity:
    """interface_states.jl:160-185: q_s = beta q_sat(T_s); efficiency a number or CriticalSaturation."""
    efficiency: object = field(default_factory=CriticalSaturation)
    phase: str = "liquid"


@dataclass
class SkinHumidity:
    """interface_states.jl:187-229, 600-651: q_s from the soil vapor-flux balance."""
    surface_thickness: float = 0.01
    vapor_diffusivity: float = 2.5e-5
    phase: str = "liquid"


@dataclass
class StorageBasedDryLayerDepth:
    """dry_layer_humidity.jl:81-100: delta(S) = delta_max (1 - min(S / S_c, 1))^eta."""
    maximum_dry_layer_depth: float
    dry_layer_onset_saturation: float
    dry_layer_exponent: float = 2.0


class ConstantTortuosity:
    """dry_layer_humidity.jl:111-118, 255-256: D_eff = D_0."""


class PowerLawTortuosity:
    """dry_layer_humidity.jl:120-127, 258-263: D_eff = D_0 theta_g^(10/3) / nu^2 (Millington-Quirk)."""


@dataclass
class DryLayerVaporPistonVelocity:
    """dry_layer_humidity.jl:155-167 (wet_transition_width None = 5 minimum_dry_layer_depth)."""
    minimum_dry_layer_depth: float
    molecular_diffusivity: float
    wet_transition_width: Optional[float] = None
    tortuosity: object = field(default_factory=ConstantTortuosity)

    def __post_init__(self):
        if self.wet_transition_width is None:
            self.wet_transition_width = 5 * self.minimum_dry_layer_depth


@dataclass
class DryLayerHumidity:
    """dry_layer_humidity.jl:216-235, 317-366: q_s from the vapor-flux balance across a dry
    surface layer, blended with the saturated skin."""
    dry_layer_depth: StorageBasedDryLayerDepth
    vapor_exchange: DryLayerVaporPistonVelocity
    thermal_exchange_depth: float
    porosity: float
    phase: str = "liquid"


def default_ao_specific_humidity():
    """component_interfaces.jl:353-358: Liquid with x_H2O = 0.98."""
    return ImpureSaturationSpecificHumidity("liquid", 0.98)


class BulkTemperature:
    """interface_states.jl:330-333."""


@dataclass
class ConductiveFlux:
    """ClimaSeaIce ConductiveFlux(conductivity); sea_ice_simulation.jl default conductivity = 2."""
    conductivity: float = 2.0


@dataclass
class IceSnowConductiveFlux:
    """ClimaSeaIce IceSnowConductiveFlux(snow_conductivity, ice_conductivity) (interface_states.jl:519-524)."""
    snow_conductivity: float = 0.31
    ice_conductivity: float = 2.0


@dataclass
class InteriorDiffusivity:
    """interface_states.jl:384-391."""
    minimum_diffusivity: float = 1.4e-7


@dataclass
class DiffusiveFlux:
    """interface_states.jl:371-374."""
    κ: object = 1e-2
    δ: float = 1.0


@dataclass
class SkinTemperature:
    """interface_states.jl:355-360."""
    internal_flux: object = field(default_factory=IceSnowConductiveFlux)
    max_ΔT: float = 5.0


class RelativeVelocity:
    """interface_states.jl:287,295-299."""


class WindVelocity:
    """interface_states.jl:284,301."""


@dataclass
class LinearLiquidus:
    """ClimaSeaIce LinearLiquidus: T_m = freshwater_melting_temperature - slope * S (Celsius)."""
    freshwater_melting_temperature: float = 0.0
    slope: float = 0.054

    def melting_temperature(self, S):
        return self.freshwater_melting_temperature - self.slope * S


@dataclass
class SurfaceRadiationProperties:
    """Radiations: albedo and emissivity of one surface (prescribed_radiation.jl:53-54)."""
    albedo: float
    emissivity: float


@dataclass
class InterfaceSpec:
    """Everything the flux kernel of one interface needs: the flux formulation, the
    InterfaceProperties (interface_states.jl:8-12), atmosphere properties
    (atmosphere_ocean_fluxes.jl:8-10) and the interior properties of the surface."""
    flux_formulation: object = field(default_factory=SimilarityTheoryFluxes)   # or CoefficientBasedFluxes
    specific_humidity: ImpureSaturationSpecificHumidity = field(default_factory=default_ao_specific_humidity)
    temperature: object = field(default_factory=BulkTemperature)
    velocity: object = field(default_factory=RelativeVelocity)
    thermodynamics_parameters: AtmosphereThermodynamicsParameters = field(
        default_factory=AtmosphereThermodynamicsParameters)
    gravitational_acceleration: float = default_gravitational_acceleration
    surface_layer_height: float = 10.0          # prescribed_atmosphere.jl:222
    boundary_layer_height: float = 512.0        # prescribed_atmosphere.jl:223
    interior_temperature_units: str = "celsius"
    interface_temperature_units: str = "celsius"
    radiation: Optional[SurfaceRadiationProperties] = None
    stefan_boltzmann_constant: float = default_stefan_boltzmann_constant
    liquidus: LinearLiquidus = field(default_factory=LinearLiquidus)
    interior_reference_density: float = 1020.0
    interior_heat_capacity: float = 3991.86795711963   # TEOS-10 reference c_p (ocean_simulation.jl:527-530)

    def to_c(self):
        p = A.InterfaceParams()
        if isinstance(self.flux_formulation, CoefficientBasedFluxes):
            p.fluxes = SimilarityTheoryFluxes().to_c()   # unused by the coefficient-based iteration
            p.flux_formulation = A.FLUXES_COEFFICIENT_BASED
            p.coefficients = self.flux_formulation.coefficients_to_c()
        else:
            p.fluxes = self.flux_formulation.to_c()
            p.flux_formulation = A.FLUXES_SIMILARITY_THEORY
        p.thermo = self.thermodynamics_parameters.to_c()
        q = self.specific_humidity
        p.humidity_phase = A.PHASE_ICE if q.phase == "ice" else A.PHASE_LIQUID
        x = getattr(q, "water_mole_fraction", None)
        p.has_water_mole_fraction = 0 if x is None else 1
        p.water_mole_fraction = 1.0 if x is None else float(x)
        if isinstance(q, BulkHumidity):
            p.humidity_formulation = A.HUMIDITY_BULK
            p.evaporation_efficiency = 1.0
        elif isinstance(q, FractionalHumidity):
            p.humidity_formulation = A.HUMIDITY_FRACTIONAL
            if isinstance(q.efficiency, CriticalSaturation):
                p.critical_saturation = q.efficiency.critical_saturation
            else:
                p.evaporation_efficiency = float(q.efficiency)
        elif isinstance(q, SkinHumidity):
            p.humidity_formulation = A.HUMIDITY_SKIN
            p.skin_surface_thickness = q.surface_thickness
            p.skin_vapor_diffusivity = q.vapor_diffusivity
        elif isinstance(q, DryLayerHumidity):
            p.humidity_formulation = A.HUMIDITY_DRY_LAYER
            d, v = q.dry_layer_depth, q.vapor_exchange
            p.maximum_dry_layer_depth = d.maximum_dry_layer_depth
            p.dry_layer_onset_saturation = d.dry_layer_onset_saturation
            p.dry_layer_exponent = d.dry_layer_exponent
            p.minimum_dry_layer_depth = v.minimum_dry_layer_depth
            p.molecular_diffusivity = v.molecular_diffusivity
            p.wet_transition_width = v.wet_transition_width
            p.tortuosity = A.TORTUOSITY_POWER_LAW if isinstance(v.tortuosity, PowerLawTortuosity) \
                else A.TORTUOSITY_CONSTANT
            p.thermal_exchange_depth = q.thermal_exchange_depth
            p.porosity = q.porosity
        else:
            p.humidity_formulation = A.HUMIDITY_IMPURE_SATURATION
        p.velocity_formulation = A.WIND_VELOCITY if isinstance(self.velocity, WindVelocity) else A.RELATIVE_VELOCITY
        t = self.temperature
        p.max_delta_T = 5.0
        if isinstance(t, SkinTemperature):
            p.max_delta_T = t.max_ΔT
            f = t.internal_flux
            if isinstance(f, IceSnowConductiveFlux):
                p.temperature_formulation = A.SKIN_TEMPERATURE_CONDUCTIVE
                p.ice_conductivity = f.ice_conductivity
                p.snow_conductivity = f.snow_conductivity
            elif isinstance(f, ConductiveFlux):
                p.temperature_formulation = A.SKIN_TEMPERATURE_CONDUCTIVE
                p.ice_conductivity = f.conductivity
                p.snow_conductivity = 0.0
            elif isinstance(f, DiffusiveFlux):
                p.temperature_formulation = A.SKIN_TEMPERATURE_DIFFUSIVE
                k = f.κ
                p.diffusive_kappa = k.minimum_diffusivity if isinstance(k, InteriorDiffusivity) else float(k)
                p.diffusive_delta = f.δ
            else:
                raise NotImplementedError(type(f).__name__)
        else:
            p.temperature_formulation = A.BULK_TEMPERATURE
        p.gravitational_acceleration = self.gravitational_acceleration
        p.surface_layer_height = self.surface_layer_height
        p.boundary_layer_height = self.boundary_layer_height
        p.interior_temperature_offset = celsius_to_kelvin if self.interior_temperature_units == "celsius" else 0.0
        p.interface_temperature_offset = celsius_to_kelvin if self.interface_temperature_units == "celsius" else 0.0
        p.has_radiation = 0 if self.radiation is None else 1
        p.stefan_boltzmann_constant = self.stefan_boltzmann_constant
        if self.radiation is not None:
            p.albedo = self.radiation.albedo
            p.emissivity = self.radiation.emissivity
        p.liquidus_freshwater_melting_temperature = self.liquidus.freshwater_melting_temperature
        p.liquidus_slope = self.liquidus.slope
        p.interior_reference_density = self.interior_reference_density
        p.interior_heat_capacity = self.interior_heat_capacity
        return p


def atmosphere_ocean_interface_spec(**kw):
    """ComponentInterfaces defaults for the atmosphere-ocean interface
    (component_interfaces.jl:411-414): SimilarityTheoryFluxes, BulkTemperature,
    RelativeVelocity, ImpureSaturationSpecificHumidity(Liquid, 0.98)."""
    return InterfaceSpec(**kw)


def default_atmosphere_land_fluxes(**kw):
    """component_interfaces.jl:514-521: SimilarityTheoryFluxes with the Large-Yeager
    stability functions and constant roughness lengths (0.1 m momentum, 0.01 m scalars)."""
    kw.setdefault("stability_functions", large_yeager_stability_functions())
    kw.setdefault("momentum_roughness_length", 0.1)
    kw.setdefault("temperature_roughness_length", 0.01)
    kw.setdefault("water_vapor_roughness_length", 0.01)
    return SimilarityTheoryFluxes(**kw)


def atmosphere_land_interface_spec(**kw):
    """atmosphere_land_interface defaults (atmosphere_land_fluxes.jl:28-37,
    component_interfaces.jl:404-406, 501-521): default_atmosphere_land_fluxes,
    BulkTemperature, RelativeVelocity, BulkHumidity(Liquid); land temperatures in kelvin."""
    kw.setdefault("flux_formulation", default_atmosphere_land_fluxes())
    kw.setdefault("specific_humidity", BulkHumidity())
    kw.setdefault("interior_temperature_units", "kelvin")
    kw.setdefault("interface_temperature_units", "kelvin")
    return InterfaceSpec(**kw)


def atmosphere_sea_ice_interface_spec(**kw):
    """ComponentInterfaces defaults for the atmosphere-sea-ice interface
    (component_interfaces.jl:267-290, 412, 416; sea_ice_simulation.jl:240-249):
    Paulson/SHEBA stability, SkinTemperature(IceSnowConductiveFlux(0.31, 2)),
    ImpureSaturationSpecificHumidity(Ice), sea-ice radiation (0.7, 1.0)."""
    kw.setdefault("flux_formulation", atmosphere_sea_ice_similarity_theory())
    kw.setdefault("specific_humidity", ImpureSaturationSpecificHumidity("ice", None))
    kw.setdefault("temperature", SkinTemperature(IceSnowConductiveFlux()))
    kw.setdefault("radiation", SurfaceRadiationProperties(0.7, 1.0))
    return InterfaceSpec(**kw)


# ------------------------------------------------------------- sea ice - ocean
@dataclass
class ThreeEquationHeatFlux:
    """sea_ice_ocean_heat_flux_formulations.jl:118-159,250-260 (conductive=True is the
    ConductiveFlux variant built from the sea-ice model, sea_ice_simulation.jl:252-265)."""
    heat_transfer_coefficient: float = 0.0095
    salt_transfer_coefficient: Optional[float] = None
    friction_velocity: float = 0.002
    conductive: bool = True
    conductivity: float = 2.0

    def __post_init__(self):
        if self.salt_transfer_coefficient is None:
            self.salt_transfer_coefficient = self.heat_transfer_coefficient / 35


@dataclass
class IceBathHeatFlux:
    """sea_ice_ocean_heat_flux_formulations.jl:45-67."""
    heat_transfer_coefficient: float = 0.006
    friction_velocity: float = 0.02


@dataclass
class SeaIceOceanSpec:
    heat_flux: object = field(default_factory=ThreeEquationHeatFlux)
    reference_latent_heat: float = 334e3
    liquidus: LinearLiquidus = field(default_factory=LinearLiquidus)
    ocean_reference_density: float = 1020.0
    ocean_heat_capacity: float = 3991.86795711963
    dt: float = 300.0      # sea_ice_simulation default Δt = 5 minutes

    def to_c(self, nz=1, stride_k=0):
        p = A.IOParams()
        hf = self.heat_flux
        if isinstance(hf, IceBathHeatFlux):
            p.formulation = 1
            p.conductive = 0
            p.heat_transfer_coefficient = hf.heat_transfer_coefficient
            p.friction_velocity = hf.friction_velocity
        else:
            p.formulation = 0
            p.conductive = 1 if hf.conductive else 0
            p.heat_transfer_coefficient = hf.heat_transfer_coefficient
            p.salt_transfer_coefficient = hf.salt_transfer_coefficient
            p.friction_velocity = hf.friction_velocity
            p.ice_conductivity = hf.conductivity
        p.reference_latent_heat = self.reference_latent_heat
        p.liquidus_freshwater_melting_temperature = self.liquidus.freshwater_melting_temperature
        p.liquidus_slope = self.liquidus.slope
        p.ocean_reference_density = self.ocean_reference_density
        p.ocean_heat_capacity = self.ocean_heat_capacity
        p.dt = self.dt
        p.nz = nz
        p.stride_k = stride_k
        return p


@dataclass
class AssemblySpec:
    """Ocean/sea-ice properties used by the net-flux assembly and radiation."""
    ocean_reference_density: float = 1020.0
    ocean_heat_capacity: float = 3991.86795711963
    interface_temperature_units: str = "celsius"
    stefan_boltzmann_constant: float = default_stefan_boltzmann_constant
    ocean_surface: SurfaceRadiationProperties = field(
        default_factory=lambda: SurfaceRadiationProperties(0.05, default_water_emissivity))
    sea_ice_surface: SurfaceRadiationProperties = field(
        default_factory=lambda: SurfaceRadiationProperties(0.7, 1.0))

    def to_c(self):
        p = A.AssemblyParams()
        p.ocean_reference_density = self.ocean_reference_density
        p.ocean_heat_capacity = self.ocean_heat_capacity
        p.interface_temperature_offset = celsius_to_kelvin if self.interface_temperature_units == "celsius" else 0.0
        p.stefan_boltzmann_constant = self.stefan_boltzmann_constant
        p.ocean_albedo = self.ocean_surface.albedo
        p.ocean_emissivity = self.ocean_surface.emissivity
        p.ice_albedo = self.sea_ice_surface.albedo
        p.ice_emissivity = self.sea_ice_surface.emissivity
        return p


@dataclass
class LandRadiation:
    """The land surface of PrescribedRadiation (prescribed_radiation.jl:56, land_surface): the
    reference has no default (nothing: no land radiation); its coupled dry-layer test uses
    SurfaceRadiationProperties(0.2, 0.95)."""
    land_surface: SurfaceRadiationProperties
    stefan_boltzmann_constant: float = default_stefan_boltzmann_constant

    def to_c(self):
        p = A.LandRadiationParams()
        p.stefan_boltzmann_constant = self.stefan_boltzmann_constant
        p.land_albedo = self.land_surface.albedo
        p.land_emissivity = self.land_surface.emissivity
        return p
