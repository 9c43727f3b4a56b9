"""ctypes mirror of include/nesf.h (the C ABI of libnesf.so).

Field order and types follow the header exactly; `tests/test_abi.py` checks the
sizes against `nesf_struct_sizes` exported by the library.
"""
import ctypes as C

NESF_OK = 0
NESF_ERR_ARG = 1
NESF_ERR_NONFINITE = 2
NESF_ERR_TIMEOUT = 3
NESF_ERR_CUDA = 4
NESF_ERR_UNSUPPORTED = 5
NESF_ERR_CAPACITY = 6

NESF_F64 = 0
NESF_F32 = 1

PSI_ZERO = 0
PSI_EDSON_MOMENTUM = 1
PSI_EDSON_SCALAR = 2
PSI_SHEBA_PAULSON_MOMENTUM = 3
PSI_SHEBA_PAULSON_SCALAR = 4
PSI_LINEAR_PAULSON_MOMENTUM = 5
PSI_LINEAR_PAULSON_SCALAR = 6

ROUGHNESS_CONSTANT = 0
ROUGHNESS_MOMENTUM = 1
ROUGHNESS_SCALAR = 2

SUBGRID_NONE = 0
SUBGRID_CONSTANT = 1
SUBGRID_CONVECTIVE = 2

STOP_CONVERGENCE = 0
STOP_FIXED_ITERATIONS = 1

PROFILE_LOGARITHMIC = 0
PROFILE_COARE = 1

PHASE_LIQUID = 0
PHASE_ICE = 1

RELATIVE_VELOCITY = 0
WIND_VELOCITY = 1

BULK_TEMPERATURE = 0
SKIN_TEMPERATURE_CONDUCTIVE = 1
SKIN_TEMPERATURE_DIFFUSIVE = 2

PLAIN_F64 = 0
F32_POLISH = 1
F32_ADAPTIVE = 2

ITER_HIST_BINS = 128

vp = C.c_void_p
d = C.c_double
i32 = C.c_int32
i64 = C.c_int64


class Grid(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("hx", i32), ("hy", i32), ("stride_j", i64)]


class ThermodynamicsParameters(C.Structure):
    _fields_ = [(n, d) for n in (
        "gas_constant", "dry_air_molar_mass", "water_molar_mass", "dry_air_adiabatic_exponent",
        "water_vapor_heat_capacity", "liquid_water_heat_capacity", "water_ice_heat_capacity",
        "reference_vaporization_enthalpy", "reference_sublimation_enthalpy", "reference_temperature",
        "triple_point_temperature", "triple_point_pressure")]


class StabilityFunction(C.Structure):
    _fields_ = [("kind", i32), ("pad_", i32), ("c", d * 12)]


class RoughnessLength(C.Structure):
    _fields_ = [("kind", i32), ("wave_kind", i32), ("viscosity_kind", i32), ("pad_", i32),
                ("value", d), ("gravitational_acceleration", d), ("air_kinematic_viscosity", d),
                ("viscosity_coefficients", d * 4), ("charnock", d), ("wave_umax", d), ("wave_c1", d),
                ("wave_c2", d), ("smooth_wall_parameter", d), ("maximum_roughness_length", d),
                ("reynolds_A", d), ("reynolds_b", d)]


class SimilarityTheoryFluxesC(C.Structure):
    _fields_ = [("von_karman_constant", d), ("turbulent_prandtl_number", d),
                ("subgrid_kind", i32), ("similarity_form", i32),
                ("gustiness_parameter", d), ("minimum_gustiness", d),
                ("constant_subgrid_velocity", d), ("mesoscale_subgrid_velocity", d),
                ("stability", StabilityFunction * 3), ("roughness", RoughnessLength * 3),
                ("zero_plane_displacement", d), ("stop_kind", i32), ("maxiter", i32), ("tolerance", d)]


FLUXES_SIMILARITY_THEORY = 0
FLUXES_COEFFICIENT_BASED = 1
COEFFICIENTS_CONSTANT = 0
COEFFICIENTS_LARGE_YEAGER = 1


class CoefficientFluxes(C.Structure):
    _fields_ = [("kind", i32), ("stop_kind", i32), ("maxiter", i32), ("polynomial_mask", i32), ("tolerance", d),
                ("momentum", d), ("temperature", d), ("water_vapor", d), ("von_karman_constant", d),
                ("drag_a", d), ("drag_b", d), ("drag_c", d), ("drag_d", d), ("high_wind_speed_threshold", d),
                ("high_wind_drag_coefficient", d), ("minimum_wind_speed", d), ("reference_height", d),
                ("stable_heat_transfer_coefficient", d), ("unstable_heat_transfer_coefficient", d),
                ("moisture_transfer_coefficient", d), ("stability", StabilityFunction * 2)]


class InterfaceParams(C.Structure):
    _fields_ = [("fluxes", SimilarityTheoryFluxesC), ("thermo", ThermodynamicsParameters),
                ("humidity_phase", i32), ("has_water_mole_fraction", i32), ("water_mole_fraction", d),
                ("velocity_formulation", i32), ("temperature_formulation", i32),
                ("max_delta_T", d), ("ice_conductivity", d), ("snow_conductivity", d),
                ("diffusive_kappa", d), ("diffusive_delta", d),
                ("gravitational_acceleration", d), ("surface_layer_height", d), ("boundary_layer_height", d),
                ("interior_temperature_offset", d), ("interface_temperature_offset", d),
                ("has_radiation", i32), ("pad_", i32),
                ("stefan_boltzmann_constant", d), ("albedo", d), ("emissivity", d),
                ("liquidus_freshwater_melting_temperature", d), ("liquidus_slope", d),
                ("interior_reference_density", d), ("interior_heat_capacity", d),
                ("flux_formulation", i32), ("pad2_", i32), ("coefficients", CoefficientFluxes),
                ("humidity_formulation", i32), ("pad3_", i32), ("evaporation_efficiency", d),
                ("critical_saturation", d), ("skin_surface_thickness", d), ("skin_vapor_diffusivity", d),
                ("tortuosity", i32), ("pad4_", i32), ("maximum_dry_layer_depth", d),
                ("dry_layer_onset_saturation", d), ("dry_layer_exponent", d), ("minimum_dry_layer_depth", d),
                ("molecular_diffusivity", d), ("wet_transition_width", d), ("thermal_exchange_depth", d),
                ("porosity", d)]


class SolverOptions(C.Structure):
    _fields_ = [("precision", i32), ("polish_maxiter", i32), ("block_size", i32), ("schedule", i32),
                ("ctas_per_sm", i32), ("warm_start", i32), ("mlp", vp), ("fallback_ratio", d), ("path_tolerance", d),
                ("fp32_rho", d), ("calm_replay_wind", d)]


class Stats(C.Structure):
    _fields_ = [("cells", i64), ("solved", i64), ("iterations", i64), ("max_iterations", i64),
                ("nonconverged", i64), ("polished", i64), ("polish_iterations", i64),
                ("cold_fallbacks", i64), ("fp64_redo", i64), ("replay_reasons", i64 * 5), ("histogram", i64 * ITER_HIST_BINS)]


class AOFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in (
        "u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "u_oc", "v_oc", "T_oc", "S_oc", "inactive",
        "sw_down", "lw_down", "kappa",
        "latent_heat", "sensible_heat", "water_vapor", "x_momentum", "y_momentum",
        "friction_velocity", "temperature_scale", "water_vapor_scale", "interface_temperature",
        "iterations")]


class AIFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in (
        "u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "T_oc", "S_oc", "ice_thickness", "snow_thickness",
        "consolidation_thickness", "ice_concentration", "inactive", "sw_down", "lw_down",
        "interface_temperature", "latent_heat", "sensible_heat", "water_vapor", "x_momentum",
        "y_momentum", "iterations")]


HUMIDITY_IMPURE_SATURATION = 0
HUMIDITY_BULK = 1
HUMIDITY_FRACTIONAL = 2
HUMIDITY_SKIN = 3
HUMIDITY_DRY_LAYER = 4
TIME_CYCLICAL = 0
TIME_LINEAR = 1
TIME_CLAMP = 2
TORTUOSITY_CONSTANT = 0
TORTUOSITY_POWER_LAW = 1


class ALFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in (
        "u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "land_temperature", "saturation",
        "latent_heat", "sensible_heat", "water_vapor", "x_momentum", "y_momentum", "friction_velocity",
        "temperature_scale", "water_vapor_scale", "interface_temperature", "iterations")]


class IOParams(C.Structure):
    _fields_ = [("formulation", i32), ("conductive", i32),
                ("heat_transfer_coefficient", d), ("salt_transfer_coefficient", d),
                ("friction_velocity", d), ("ice_conductivity", d), ("reference_latent_heat", d),
                ("liquidus_freshwater_melting_temperature", d), ("liquidus_slope", d),
                ("ocean_reference_density", d), ("ocean_heat_capacity", d), ("dt", d),
                ("nz", i32), ("pad_", i32), ("stride_k", i64)]


class IOFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in (
        "T_oc", "S_oc", "dz", "ice_salinity", "ice_thickness", "consolidation_thickness",
        "ice_concentration", "internal_temperature", "ice_mass_flux", "snow_mass_flux",
        "interface_heat", "frazil_heat", "salt", "freshwater", "interface_T", "interface_S")]


class AtmosGrid(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("hx", i32), ("hy", i32), ("stride_j", i64), ("stride_t", i64),
                ("lon0", d), ("dlon", d), ("lat0", d), ("dlat", d)]


class ExchangeCoords(C.Structure):
    _fields_ = [("lon0", d), ("dlon", d), ("lat0", d), ("dlat", d)]


class InterpFields(C.Structure):
    _fields_ = [("grid", Grid), ("coords", ExchangeCoords), ("atmos", AtmosGrid), ("dtype", i32),
                ("pad_", i32), ("time_weight", d)] + [(n, vp) for n in (
        "u", "v", "T", "q", "p", "rain", "snow", "sw_down", "lw_down",
        "u_out", "v_out", "T_out", "q_out", "p_out", "rain_out", "snow_out", "sw_out", "lw_out",
        "frac_i", "frac_j")]


class AssemblyParams(C.Structure):
    _fields_ = [(n, d) for n in (
        "ocean_reference_density", "ocean_heat_capacity", "interface_temperature_offset",
        "stefan_boltzmann_constant", "ocean_albedo", "ocean_emissivity", "ice_albedo", "ice_emissivity")]


ASSEMBLY_FIELD_NAMES = (
    "inactive", "ice_concentration", "ocean_surface_temperature", "rain", "snow", "intercepted_snow",
    "land_freshwater", "ao_sensible", "ao_latent", "ao_water_vapor", "ao_x_momentum", "ao_y_momentum",
    "ao_interface_temperature", "io_interface_heat", "io_frazil_heat", "io_salt", "io_freshwater",
    "io_x_momentum", "io_y_momentum", "ai_sensible", "ai_latent", "ai_x_momentum", "ai_y_momentum",
    "ai_interface_temperature", "sw_down", "lw_down",
    "ocean_u", "ocean_v", "ocean_T", "ocean_S", "ocean_eta", "ocean_heat_content",
    "ice_top_heat", "ice_top_snowfall", "ice_top_u", "ice_top_v", "ice_bottom_heat",
    "ocean_upwelling_longwave", "ocean_downwelling_longwave", "ocean_downwelling_shortwave",
    "ice_upwelling_longwave", "ice_downwelling_longwave", "ice_downwelling_shortwave")


class AssemblyFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in ASSEMBLY_FIELD_NAMES]


class LandRadiationParams(C.Structure):
    _fields_ = [("stefan_boltzmann_constant", d), ("land_albedo", d), ("land_emissivity", d)]


LAND_FLUX_FIELD_NAMES = (
    "inactive", "rain", "al_sensible", "al_latent", "al_water_vapor", "al_interface_temperature",
    "sw_down", "lw_down", "surface_energy_flux", "precipitation", "evaporation", "vapor_flux",
    "liquid_precipitation_flux", "upwelling_longwave", "downwelling_longwave", "downwelling_shortwave")


class LandFluxFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("pad_", i32)] + [(n, vp) for n in LAND_FLUX_FIELD_NAMES]


class CouplingStepArgs(C.Structure):
    _fields_ = [("ao_params", C.POINTER(InterfaceParams)), ("ao", C.POINTER(AOFields)),
                ("ai_params", C.POINTER(InterfaceParams)), ("ai", C.POINTER(AIFields)),
                ("io_params", C.POINTER(IOParams)), ("io", C.POINTER(IOFields)),
                ("interp", C.POINTER(InterpFields)),
                ("assembly_params", C.POINTER(AssemblyParams)), ("assembly", C.POINTER(AssemblyFields)),
                ("radiation", i32), ("pad_", i32)]


class MlpTrainOptions(C.Structure):
    _fields_ = [("epochs", i32), ("batch", i32), ("learning_rate", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float)]


# the warm-start network's device blob (nesf_mlp.cuh, struct Blob)
MLP_IN, MLP_IN_PAD, MLP_HID, MLP_OUT, MLP_OUT_PAD = 6, 16, 64, 3, 16
MLP_W1 = 0
MLP_B1 = MLP_W1 + MLP_HID * MLP_IN_PAD
MLP_W2 = MLP_B1 + MLP_HID
MLP_B2 = MLP_W2 + MLP_HID * MLP_HID
MLP_W3 = MLP_B2 + MLP_HID
MLP_B3 = MLP_W3 + MLP_OUT_PAD * MLP_HID
MLP_PARAMS = MLP_B3 + MLP_OUT_PAD


class MlpBlob(C.Structure):
    _fields_ = [("p", C.c_float * MLP_PARAMS), ("g", C.c_float * MLP_PARAMS), ("m", C.c_float * MLP_PARAMS),
                ("v", C.c_float * MLP_PARAMS), ("in_mu", C.c_float * 8), ("in_sig", C.c_float * 8),
                ("out_mu", C.c_float * 4), ("out_sig", C.c_float * 4), ("loss", C.c_float * 4), ("steps", i32),
                ("error", i32), ("pad_", i32 * 2), ("stats", C.c_double * 32),
                ("w1h", C.c_uint16 * (MLP_HID * MLP_IN_PAD)), ("w2h", C.c_uint16 * (MLP_HID * MLP_HID)),
                ("w3h", C.c_uint16 * (MLP_OUT_PAD * MLP_HID))]


MAX_INTEGRALS = 16


class IntegralFields(C.Structure):
    _fields_ = [("grid", Grid), ("dtype", i32), ("n", i32), ("field", vp * MAX_INTEGRALS),
                ("factor", vp * MAX_INTEGRALS), ("inactive", vp), ("area", vp), ("row_area", vp),
                ("uniform_area", d)]


class Tuning(C.Structure):
    _fields_ = [("solve_block", i32), ("deferred_per_sm", i32), ("infer_per_sm", i32), ("two_lanes", i32),
                ("io_overlap", i32), ("pass1_fetch", i32), ("refill_lanes", i32), ("early_ocean_classify", i32),
                ("ice_deferred_per_sm", i32), ("cells_per_thread", i32), ("step_ms", d)]


TUNING_FIELDS = ("solve_block", "deferred_per_sm", "infer_per_sm", "two_lanes", "io_overlap", "pass1_fetch",
                 "refill_lanes", "early_ocean_classify", "ice_deferred_per_sm", "cells_per_thread")

TUNING_VERSION = 2


class TuningKey(C.Structure):
    _fields_ = [("device", C.c_char * 64), ("sm_count", i32), ("compute_capability", i32), ("nx", i32), ("ny", i32),
                ("hx", i32), ("hy", i32), ("dtype", i32), ("precision", i32), ("warm_start", i32), ("parts", i32),
                ("flux_formulation", i32)]


TRACE_MAX = 64

# NESF_WORK_* of include/nesf.h (checked against the header by the tests)
WORK = {"ITER_TRANSCENDENTALS": 55, "ITER_FLOPS": 300, "PROLOGUE_TRANSCENDENTALS": 2, "PROLOGUE_FLOPS": 20,
        "EPILOGUE_TRANSCENDENTALS": 1, "EPILOGUE_FLOPS": 35, "BYTES_PER_CELL_F32": 72}


class TraceEntry(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("stream", i32), ("pad_", i32), ("t_ms", d)]


# Order of nesf_struct_sizes(): must match the library.
STRUCTS_IN_SIZE_ORDER = (Grid, ThermodynamicsParameters, StabilityFunction, RoughnessLength,
                         SimilarityTheoryFluxesC, InterfaceParams, SolverOptions, Stats, AOFields,
                         AIFields, IOParams, IOFields, AtmosGrid, ExchangeCoords, InterpFields,
                         AssemblyParams, AssemblyFields, CouplingStepArgs, IntegralFields, Tuning,
                         TraceEntry, CoefficientFluxes, ALFields, LandRadiationParams, LandFluxFields, TuningKey)
