# NESF.jl -- the binding that routes NumericalEarth.jl's interface-flux step to
# libnesf.so through `ccall`. Not executed in this repository (there is no Julia
# toolchain here): it is the binding a NumericalEarth maintainer would add, written
# against include/nesf.h. The Python tests check every struct mirror below against
# the header's layout (offsetof) and every `ccall`'s argument list against the
# header's prototype (tests/test_julia_shim.py).
#
# Usage: wrap the atmosphere-ocean flux formulation; the whole interface-flux step of
# update_state! (time_step_earth_system_model.jl:38-83) then runs through the library:
#
#     using NumericalEarth, NESF
#     fluxes = NESF.GB300SimilarityTheoryFluxes(SimilarityTheoryFluxes(); precision = :f32_adaptive)
#     interfaces = ComponentInterfaces(atmosphere, ocean, sea_ice; radiation,
#                                      atmosphere_ocean_fluxes = fluxes)
#     coupled_model = EarthSystemModel(atmosphere, ocean, sea_ice; radiation, interfaces)
#
# update_state! calls each phase with the coupled model alone (`f(coupled_model)` or
# `f(coupled_model, component)`); the methods below are specialised on the model type
# whose ComponentInterfaces carry the wrapper (GB300Model), so Julia's dispatch picks
# them over the reference's generic ones. Each method packs the reference's own objects
# (flux formulations, interface properties, thermodynamics parameters, the atmosphere's
# heights, the ocean and sea-ice properties) into the library's parameter structs and
# passes the device pointers of the Oceananigans fields (parent arrays: halo included,
# i fastest). A formulation the library does not implement falls back to the reference's
# own method (`invoke` of the generic method).
module NESF

using CUDA
using Oceananigans
using Oceananigans: architecture
using Oceananigans.Grids: halo_size
using Oceananigans.OutputReaders: FieldTimeSeries
using NumericalEarth
using NumericalEarth.EarthSystemModels: EarthSystemModels, EarthSystemModel
using NumericalEarth.EarthSystemModels.InterfaceComputations: InterfaceComputations
using NumericalEarth.Atmospheres: PrescribedAtmosphere, boundary_layer_height, thermodynamics_parameters
using ClimaSeaIce: SeaIceModel
const IC = InterfaceComputations
const ESM = EarthSystemModels

const libnesf = get(ENV, "NESF_LIB", joinpath(@__DIR__, "..", "nesf", "libnesf.so"))

# ----------------------------------------------------------- constants (nesf.h)
const NESF_OK = Cint(0)
const NESF_F64 = Int32(0)
const NESF_F32 = Int32(1)
const NESF_PLAIN_F64 = Int32(0)
const NESF_F32_POLISH = Int32(1)
const NESF_F32_ADAPTIVE = Int32(2)
const PSI_ZERO, PSI_EDSON_MOMENTUM, PSI_EDSON_SCALAR = Int32(0), Int32(1), Int32(2)
const PSI_SHEBA_PAULSON_MOMENTUM, PSI_SHEBA_PAULSON_SCALAR = Int32(3), Int32(4)
const PSI_LINEAR_PAULSON_MOMENTUM, PSI_LINEAR_PAULSON_SCALAR = Int32(5), Int32(6)
const ROUGHNESS_CONSTANT, ROUGHNESS_MOMENTUM, ROUGHNESS_SCALAR = Int32(0), Int32(1), Int32(2)
const SUBGRID_NONE, SUBGRID_CONSTANT, SUBGRID_CONVECTIVE = Int32(0), Int32(1), Int32(2)
const STOP_CONVERGENCE, STOP_FIXED_ITERATIONS = Int32(0), Int32(1)
const PROFILE_LOGARITHMIC, PROFILE_COARE = Int32(0), Int32(1)
const PHASE_LIQUID, PHASE_ICE = Int32(0), Int32(1)
const RELATIVE_VELOCITY, WIND_VELOCITY = Int32(0), Int32(1)
const BULK_TEMPERATURE, SKIN_TEMPERATURE_CONDUCTIVE, SKIN_TEMPERATURE_DIFFUSIVE = Int32(0), Int32(1), Int32(2)
const FLUXES_SIMILARITY_THEORY = Int32(0)

# --------------------------------------------------------- struct mirrors (nesf.h)
# isbits structs laid out as the C structs (Julia uses the C layout rules for them).
struct Grid
    nx::Int32; ny::Int32; hx::Int32; hy::Int32; stride_j::Int64
end

struct ThermodynamicsParameters
    gas_constant::Float64; dry_air_molar_mass::Float64; water_molar_mass::Float64
    dry_air_adiabatic_exponent::Float64; water_vapor_heat_capacity::Float64
    liquid_water_heat_capacity::Float64; water_ice_heat_capacity::Float64
    reference_vaporization_enthalpy::Float64; reference_sublimation_enthalpy::Float64
    reference_temperature::Float64; triple_point_temperature::Float64; triple_point_pressure::Float64
end

struct StabilityFunction
    kind::Int32; pad_::Int32; c::NTuple{12, Float64}
end

struct RoughnessLength
    kind::Int32; wave_kind::Int32; viscosity_kind::Int32; pad_::Int32
    value::Float64; gravitational_acceleration::Float64; air_kinematic_viscosity::Float64
    viscosity_coefficients::NTuple{4, Float64}
    charnock::Float64; wave_umax::Float64; wave_c1::Float64; wave_c2::Float64
    smooth_wall_parameter::Float64; maximum_roughness_length::Float64
    reynolds_A::Float64; reynolds_b::Float64
end

struct SimilarityTheoryFluxesC
    von_karman_constant::Float64; turbulent_prandtl_number::Float64
    subgrid_kind::Int32; similarity_form::Int32
    gustiness_parameter::Float64; minimum_gustiness::Float64
    constant_subgrid_velocity::Float64; mesoscale_subgrid_velocity::Float64
    stability::NTuple{3, StabilityFunction}
    roughness::NTuple{3, RoughnessLength}
    zero_plane_displacement::Float64
    stop_kind::Int32; maxiter::Int32
    tolerance::Float64
end

struct CoefficientFluxes
    kind::Int32; stop_kind::Int32; maxiter::Int32; polynomial_mask::Int32
    tolerance::Float64; momentum::Float64; temperature::Float64; water_vapor::Float64
    von_karman_constant::Float64; drag_a::Float64; drag_b::Float64; drag_c::Float64; drag_d::Float64
    high_wind_speed_threshold::Float64; high_wind_drag_coefficient::Float64; minimum_wind_speed::Float64
    reference_height::Float64; stable_heat_transfer_coefficient::Float64
    unstable_heat_transfer_coefficient::Float64; moisture_transfer_coefficient::Float64
    stability::NTuple{2, StabilityFunction}
end

struct InterfaceParams
    fluxes::SimilarityTheoryFluxesC
    thermo::ThermodynamicsParameters
    humidity_phase::Int32; has_water_mole_fraction::Int32
    water_mole_fraction::Float64
    velocity_formulation::Int32; temperature_formulation::Int32
    max_delta_T::Float64; ice_conductivity::Float64; snow_conductivity::Float64
    diffusive_kappa::Float64; diffusive_delta::Float64
    gravitational_acceleration::Float64; surface_layer_height::Float64; boundary_layer_height::Float64
    interior_temperature_offset::Float64; interface_temperature_offset::Float64
    has_radiation::Int32; pad_::Int32
    stefan_boltzmann_constant::Float64; albedo::Float64; emissivity::Float64
    liquidus_freshwater_melting_temperature::Float64; liquidus_slope::Float64
    interior_reference_density::Float64; interior_heat_capacity::Float64
    flux_formulation::Int32; pad2_::Int32
    coefficients::CoefficientFluxes
    humidity_formulation::Int32; pad3_::Int32
    evaporation_efficiency::Float64; critical_saturation::Float64
    skin_surface_thickness::Float64; skin_vapor_diffusivity::Float64
    tortuosity::Int32; pad4_::Int32
    maximum_dry_layer_depth::Float64; dry_layer_onset_saturation::Float64; dry_layer_exponent::Float64
    minimum_dry_layer_depth::Float64; molecular_diffusivity::Float64; wet_transition_width::Float64
    thermal_exchange_depth::Float64; porosity::Float64
end

struct SolverOptions
    precision::Int32; polish_maxiter::Int32; block_size::Int32; schedule::Int32
    ctas_per_sm::Int32; warm_start::Int32; mlp::Ptr{Cvoid}
    fallback_ratio::Float64; path_tolerance::Float64; fp32_rho::Float64; calm_replay_wind::Float64
end

struct AOFields
    grid::Grid; dtype::Int32; pad_::Int32
    u_atm::Ptr{Cvoid}; v_atm::Ptr{Cvoid}; T_atm::Ptr{Cvoid}; p_atm::Ptr{Cvoid}; q_atm::Ptr{Cvoid}
    u_oc::Ptr{Cvoid}; v_oc::Ptr{Cvoid}; T_oc::Ptr{Cvoid}; S_oc::Ptr{Cvoid}; inactive::Ptr{UInt8}
    sw_down::Ptr{Cvoid}; lw_down::Ptr{Cvoid}; kappa::Ptr{Cvoid}
    latent_heat::Ptr{Cvoid}; sensible_heat::Ptr{Cvoid}; water_vapor::Ptr{Cvoid}
    x_momentum::Ptr{Cvoid}; y_momentum::Ptr{Cvoid}
    friction_velocity::Ptr{Cvoid}; temperature_scale::Ptr{Cvoid}; water_vapor_scale::Ptr{Cvoid}
    interface_temperature::Ptr{Cvoid}; iterations::Ptr{Int32}
end

struct ALFields
    grid::Grid; dtype::Int32; pad_::Int32
    u_atm::Ptr{Cvoid}; v_atm::Ptr{Cvoid}; T_atm::Ptr{Cvoid}; p_atm::Ptr{Cvoid}; q_atm::Ptr{Cvoid}
    land_temperature::Ptr{Cvoid}; saturation::Ptr{Cvoid}
    latent_heat::Ptr{Cvoid}; sensible_heat::Ptr{Cvoid}; water_vapor::Ptr{Cvoid}
    x_momentum::Ptr{Cvoid}; y_momentum::Ptr{Cvoid}
    friction_velocity::Ptr{Cvoid}; temperature_scale::Ptr{Cvoid}; water_vapor_scale::Ptr{Cvoid}
    interface_temperature::Ptr{Cvoid}; iterations::Ptr{Int32}
end

struct AIFields
    grid::Grid; dtype::Int32; pad_::Int32
    u_atm::Ptr{Cvoid}; v_atm::Ptr{Cvoid}; T_atm::Ptr{Cvoid}; p_atm::Ptr{Cvoid}; q_atm::Ptr{Cvoid}
    T_oc::Ptr{Cvoid}; S_oc::Ptr{Cvoid}
    ice_thickness::Ptr{Cvoid}; snow_thickness::Ptr{Cvoid}; consolidation_thickness::Ptr{Cvoid}
    ice_concentration::Ptr{Cvoid}; inactive::Ptr{UInt8}
    sw_down::Ptr{Cvoid}; lw_down::Ptr{Cvoid}
    interface_temperature::Ptr{Cvoid}
    latent_heat::Ptr{Cvoid}; sensible_heat::Ptr{Cvoid}; water_vapor::Ptr{Cvoid}
    x_momentum::Ptr{Cvoid}; y_momentum::Ptr{Cvoid}
    iterations::Ptr{Int32}
end

struct IOParams
    formulation::Int32; conductive::Int32
    heat_transfer_coefficient::Float64; salt_transfer_coefficient::Float64; friction_velocity::Float64
    ice_conductivity::Float64; reference_latent_heat::Float64
    liquidus_freshwater_melting_temperature::Float64; liquidus_slope::Float64
    ocean_reference_density::Float64; ocean_heat_capacity::Float64; dt::Float64
    nz::Int32; pad_::Int32; stride_k::Int64
end

struct IOFields
    grid::Grid; dtype::Int32; pad_::Int32
    T_oc::Ptr{Cvoid}; S_oc::Ptr{Cvoid}; dz::Ptr{Float64}
    ice_salinity::Ptr{Cvoid}; ice_thickness::Ptr{Cvoid}; consolidation_thickness::Ptr{Cvoid}
    ice_concentration::Ptr{Cvoid}; internal_temperature::Ptr{Cvoid}
    ice_mass_flux::Ptr{Cvoid}; snow_mass_flux::Ptr{Cvoid}
    interface_heat::Ptr{Cvoid}; frazil_heat::Ptr{Cvoid}; salt::Ptr{Cvoid}; freshwater::Ptr{Cvoid}
    interface_T::Ptr{Cvoid}; interface_S::Ptr{Cvoid}
end

struct AtmosGrid
    nx::Int32; ny::Int32; hx::Int32; hy::Int32
    stride_j::Int64; stride_t::Int64
    lon0::Float64; dlon::Float64; lat0::Float64; dlat::Float64
end

struct ExchangeCoords
    lon0::Float64; dlon::Float64; lat0::Float64; dlat::Float64
end

struct InterpFields
    grid::Grid; coords::ExchangeCoords; atmos::AtmosGrid
    dtype::Int32; pad_::Int32
    time_weight::Float64
    u::Ptr{Cvoid}; v::Ptr{Cvoid}; T::Ptr{Cvoid}; q::Ptr{Cvoid}; p::Ptr{Cvoid}
    rain::Ptr{Cvoid}; snow::Ptr{Cvoid}; sw_down::Ptr{Cvoid}; lw_down::Ptr{Cvoid}
    u_out::Ptr{Cvoid}; v_out::Ptr{Cvoid}; T_out::Ptr{Cvoid}; q_out::Ptr{Cvoid}; p_out::Ptr{Cvoid}
    rain_out::Ptr{Cvoid}; snow_out::Ptr{Cvoid}; sw_out::Ptr{Cvoid}; lw_out::Ptr{Cvoid}
    frac_i::Ptr{Float64}; frac_j::Ptr{Float64}
end

struct AssemblyParams
    ocean_reference_density::Float64; ocean_heat_capacity::Float64
    interface_temperature_offset::Float64; stefan_boltzmann_constant::Float64
    ocean_albedo::Float64; ocean_emissivity::Float64; ice_albedo::Float64; ice_emissivity::Float64
end

struct AssemblyFields
    grid::Grid; dtype::Int32; pad_::Int32
    inactive::Ptr{UInt8}; ice_concentration::Ptr{Cvoid}; ocean_surface_temperature::Ptr{Cvoid}
    rain::Ptr{Cvoid}; snow::Ptr{Cvoid}; intercepted_snow::Ptr{Cvoid}; land_freshwater::Ptr{Cvoid}
    ao_sensible::Ptr{Cvoid}; ao_latent::Ptr{Cvoid}; ao_water_vapor::Ptr{Cvoid}
    ao_x_momentum::Ptr{Cvoid}; ao_y_momentum::Ptr{Cvoid}; ao_interface_temperature::Ptr{Cvoid}
    io_interface_heat::Ptr{Cvoid}; io_frazil_heat::Ptr{Cvoid}; io_salt::Ptr{Cvoid}
    io_freshwater::Ptr{Cvoid}; io_x_momentum::Ptr{Cvoid}; io_y_momentum::Ptr{Cvoid}
    ai_sensible::Ptr{Cvoid}; ai_latent::Ptr{Cvoid}; ai_x_momentum::Ptr{Cvoid}; ai_y_momentum::Ptr{Cvoid}
    ai_interface_temperature::Ptr{Cvoid}
    sw_down::Ptr{Cvoid}; lw_down::Ptr{Cvoid}
    ocean_u::Ptr{Cvoid}; ocean_v::Ptr{Cvoid}; ocean_T::Ptr{Cvoid}; ocean_S::Ptr{Cvoid}
    ocean_eta::Ptr{Cvoid}; ocean_heat_content::Ptr{Cvoid}
    ice_top_heat::Ptr{Cvoid}; ice_top_snowfall::Ptr{Cvoid}; ice_top_u::Ptr{Cvoid}; ice_top_v::Ptr{Cvoid}
    ice_bottom_heat::Ptr{Cvoid}
    ocean_upwelling_longwave::Ptr{Cvoid}; ocean_downwelling_longwave::Ptr{Cvoid}
    ocean_downwelling_shortwave::Ptr{Cvoid}; ice_upwelling_longwave::Ptr{Cvoid}
    ice_downwelling_longwave::Ptr{Cvoid}; ice_downwelling_shortwave::Ptr{Cvoid}
end

# ---------------------------------------------------------------- the wrapper
struct GB300SimilarityTheoryFluxes{F}
    inner :: F          # the reference's formulation, packed field by field
    precision :: Symbol # :f64 (the drop-in), :f32 (FP32 sweep + FP64 Newton polish) or
                        # :f32_adaptive (FP32 result kept where well conditioned)
end
GB300SimilarityTheoryFluxes(inner; precision = :f64) = GB300SimilarityTheoryFluxes(inner, precision)
Base.summary(f::GB300SimilarityTheoryFluxes) = "GB300SimilarityTheoryFluxes($(summary(f.inner)), $(f.precision))"
Base.show(io::IO, f::GB300SimilarityTheoryFluxes) = print(io, summary(f))

# The coupled models whose atmosphere-ocean flux formulation is the wrapper:
# EarthSystemModel{R, A, L, I, O, F, C, Arch} with F a ComponentInterfaces{AO, ...} whose AO is
# an AtmosphereInterface{J, F, ST, P} with F the wrapper (earth_system_model.jl:6,
# component_interfaces.jl:22,203).
const GB300AOInterface = IC.AtmosphereInterface{<:Any, <:GB300SimilarityTheoryFluxes}
const GB300Interfaces = IC.ComponentInterfaces{<:GB300AOInterface}
const GB300Model = EarthSystemModel{<:Any, <:Any, <:Any, <:Any, <:Any, <:GB300Interfaces}

unwrap(f::GB300SimilarityTheoryFluxes) = f.inner
unwrap(f) = f
precision_code(f::GB300SimilarityTheoryFluxes) = f.precision === :f32 ? NESF_F32_POLISH :
                                                  f.precision === :f32_adaptive ? NESF_F32_ADAPTIVE : NESF_PLAIN_F64
solver_options(model::GB300Model) =
    SolverOptions(precision_code(model.interfaces.atmosphere_ocean_interface.flux_formulation), 0, 0, 0, 0, 0,
                  C_NULL, 10.0, 2e-6, 0.9, 0.7)

# ---------------------------------------------------------------- plumbing
check(code) = code == NESF_OK ||
    error("nesf error $code: " * unsafe_string(ccall((:nesf_last_error, libnesf), Cstring, ())))

devptr(::Nothing) = C_NULL
devptr(f) = reinterpret(Ptr{Cvoid}, pointer(parent(f)))     # CuArray parent of an Oceananigans field
surface_ptr(f, k) = reinterpret(Ptr{Cvoid}, pointer(view(parent(f), :, :, k)))   # one level of a 3-D field
stream() = CUDA.stream().handle
dtype_of(grid) = eltype(grid) == Float64 ? NESF_F64 : NESF_F32

function grid_struct(grid)
    Nx, Ny, _ = size(grid)
    Hx, Hy, _ = halo_size(grid)
    return Grid(Nx, Ny, Hx, Hy, Nx + 2Hx)
end

# Write `v` at the field `path` of the struct held by `r` (names; integers index tuples).
function poke!(r::Base.RefValue{T}, path::Tuple, v) where {T}
    off = 0
    S = T
    for name in path
        i = name isa Integer ? name : findfirst(==(name), fieldnames(S))
        off += fieldoffset(S, i)
        S = fieldtype(S, i)
    end
    GC.@preserve r unsafe_store!(Ptr{S}(Base.unsafe_convert(Ptr{T}, r) + off), convert(S, v))
    return r
end

struct Unsupported <: Exception
    what :: Any
end

# ------------------------------------------ packing the reference's objects
# AtmosphereThermodynamicsParameters (thermodynamic_parameters.jl:30-181)
function pack_thermodynamics!(r, tp)
    c, h, p = tp.constitutive, tp.heat_capacity, tp.phase_transitions
    for (name, v) in ((:gas_constant, c.gas_constant), (:dry_air_molar_mass, c.dry_air_molar_mass),
                      (:water_molar_mass, c.water_molar_mass),
                      (:dry_air_adiabatic_exponent, h.dry_air_adiabatic_exponent),
                      (:water_vapor_heat_capacity, h.water_vapor_heat_capacity),
                      (:liquid_water_heat_capacity, h.liquid_water_heat_capacity),
                      (:water_ice_heat_capacity, h.water_ice_heat_capacity),
                      (:reference_vaporization_enthalpy, p.reference_vaporization_enthalpy),
                      (:reference_sublimation_enthalpy, p.reference_sublimation_enthalpy),
                      (:reference_temperature, p.reference_temperature),
                      (:triple_point_temperature, p.triple_point_temperature),
                      (:triple_point_pressure, p.triple_point_pressure))
        poke!(r, (:thermo, name), v)
    end
end

# Stability functions (similarity_theory_turbulent_fluxes.jl:487-532, 571-618, 637-752)
stability_code(::Nothing) = (PSI_ZERO, ())
stability_code(ψ::IC.EdsonMomentumStabilityFunction) =
    (PSI_EDSON_MOMENTUM, (ψ.ζmax, ψ.A⁺, ψ.B⁺, ψ.C⁺, ψ.D⁺, ψ.A⁻, ψ.B⁻, ψ.C⁻, ψ.D⁻, ψ.E⁻, ψ.F⁻))
stability_code(ψ::IC.EdsonScalarStabilityFunction) =
    (PSI_EDSON_SCALAR, (ψ.ζmax, ψ.A⁺, ψ.B⁺, ψ.C⁺, ψ.D⁺, ψ.E⁺, ψ.A⁻, ψ.B⁻, ψ.C⁻, ψ.D⁻, ψ.E⁻, ψ.F⁻))
stability_code(ψ::IC.SplitStabilityFunction{<:IC.ShebaMomentumStabilityFunction, <:IC.PaulsonMomentumStabilityFunction}) =
    (PSI_SHEBA_PAULSON_MOMENTUM, (ψ.stable.a, ψ.stable.b, ψ.unstable.a, ψ.unstable.b))
stability_code(ψ::IC.SplitStabilityFunction{<:IC.ShebaScalarStabilityFunction, <:IC.PaulsonScalarStabilityFunction}) =
    (PSI_SHEBA_PAULSON_SCALAR, (ψ.stable.a, ψ.stable.b, ψ.stable.c, ψ.unstable.a))
stability_code(ψ::IC.SplitStabilityFunction{<:IC.LinearStableStabilityFunction, <:IC.PaulsonMomentumStabilityFunction}) =
    (PSI_LINEAR_PAULSON_MOMENTUM, (ψ.stable.coefficient, ψ.stable.maximum_stability_parameter, ψ.unstable.a, ψ.unstable.b))
stability_code(ψ::IC.SplitStabilityFunction{<:IC.LinearStableStabilityFunction, <:IC.PaulsonScalarStabilityFunction}) =
    (PSI_LINEAR_PAULSON_SCALAR, (ψ.stable.coefficient, ψ.stable.maximum_stability_parameter, ψ.unstable.a))
stability_code(ψ) = throw(Unsupported(ψ))

function pack_stability!(r, path, ψ)
    kind, c = stability_code(ψ)
    poke!(r, (path..., :kind), kind)
    for (n, v) in enumerate(c)
        poke!(r, (path..., :c, n), v)
    end
end

# Roughness lengths (roughness_lengths.jl:1-246)
function pack_viscosity!(r, path, ν)
    if ν isa IC.TemperatureDependentAirViscosity
        poke!(r, (path..., :viscosity_kind), Int32(1))
        for (n, v) in enumerate((ν.ℂ₀, ν.ℂ₁, ν.ℂ₂, ν.ℂ₃))
            poke!(r, (path..., :viscosity_coefficients, n), v)
        end
    elseif ν isa Number
        poke!(r, (path..., :viscosity_kind), Int32(0))
        poke!(r, (path..., :air_kinematic_viscosity), ν)
    else
        throw(Unsupported(ν))
    end
end

function pack_roughness!(r, path, ℓ)
    if ℓ isa Number
        poke!(r, (path..., :kind), ROUGHNESS_CONSTANT)
        poke!(r, (path..., :value), ℓ)
    elseif ℓ isa IC.MomentumRoughnessLength
        poke!(r, (path..., :kind), ROUGHNESS_MOMENTUM)
        poke!(r, (path..., :gravitational_acceleration), ℓ.gravitational_acceleration)
        pack_viscosity!(r, path, ℓ.air_kinematic_viscosity)
        w = ℓ.wave_formulation
        if w isa IC.WindDependentWaveFormulation
            poke!(r, (path..., :wave_kind), Int32(1))
            poke!(r, (path..., :wave_umax), w.Umax)
            poke!(r, (path..., :wave_c1), w.ℂ₁)
            poke!(r, (path..., :wave_c2), w.ℂ₂)
        elseif w isa Number
            poke!(r, (path..., :wave_kind), Int32(0))
            poke!(r, (path..., :charnock), w)
        else
            throw(Unsupported(w))
        end
        poke!(r, (path..., :smooth_wall_parameter), ℓ.smooth_wall_parameter)
        poke!(r, (path..., :maximum_roughness_length), ℓ.maximum_roughness_length)
    elseif ℓ isa IC.ScalarRoughnessLength
        poke!(r, (path..., :kind), ROUGHNESS_SCALAR)
        pack_viscosity!(r, path, ℓ.air_kinematic_viscosity)
        poke!(r, (path..., :reynolds_A), ℓ.reynolds_number_scaling_function.A)
        poke!(r, (path..., :reynolds_b), ℓ.reynolds_number_scaling_function.b)
        poke!(r, (path..., :maximum_roughness_length), ℓ.maximum_roughness_length)
    else
        throw(Unsupported(ℓ))
    end
end

# SimilarityTheoryFluxes (similarity_theory_turbulent_fluxes.jl:9-18, 45-80, 174-214;
# compute_interface_state.jl:5-24)
function pack_fluxes!(r, f::IC.SimilarityTheoryFluxes)
    poke!(r, (:flux_formulation,), FLUXES_SIMILARITY_THEORY)
    poke!(r, (:fluxes, :von_karman_constant), f.von_karman_constant)
    poke!(r, (:fluxes, :turbulent_prandtl_number), f.turbulent_prandtl_number)
    sv, meso = f.subgrid_velocities, nothing
    if sv isa IC.SubgridVelocityCorrection
        sv, meso = sv.convective, sv.mesoscale
    end
    if sv isa IC.ConvectiveGustiness
        poke!(r, (:fluxes, :subgrid_kind), SUBGRID_CONVECTIVE)
        poke!(r, (:fluxes, :gustiness_parameter), sv.gustiness_parameter)
        poke!(r, (:fluxes, :minimum_gustiness), sv.minimum_gustiness)
    elseif sv isa Number
        poke!(r, (:fluxes, :subgrid_kind), SUBGRID_CONSTANT)
        poke!(r, (:fluxes, :constant_subgrid_velocity), sv)
    elseif isnothing(sv)
        poke!(r, (:fluxes, :subgrid_kind), SUBGRID_NONE)
    else
        throw(Unsupported(sv))
    end
    meso isa Union{Nothing, Number} || throw(Unsupported(meso))
    poke!(r, (:fluxes, :mesoscale_subgrid_velocity), isnothing(meso) ? 0.0 : meso)
    poke!(r, (:fluxes, :similarity_form),
          f.similarity_form isa IC.COARELogarithmicSimilarityProfile ? PROFILE_COARE : PROFILE_LOGARITHMIC)
    ψ = f.stability_functions
    for (n, s) in enumerate(isnothing(ψ) ? (nothing, nothing, nothing) : (ψ.momentum, ψ.temperature, ψ.water_vapor))
        pack_stability!(r, (:fluxes, :stability, n), s)
    end
    ℓ = f.roughness_lengths
    for (n, s) in enumerate((ℓ.momentum, ℓ.temperature, ℓ.water_vapor))
        pack_roughness!(r, (:fluxes, :roughness, n), s)
    end
    f.zero_plane_displacement isa Number || throw(Unsupported(f.zero_plane_displacement))
    poke!(r, (:fluxes, :zero_plane_displacement), f.zero_plane_displacement)
    sc = f.solver_stop_criteria
    if sc isa IC.FixedIterations
        poke!(r, (:fluxes, :stop_kind), STOP_FIXED_ITERATIONS)
        poke!(r, (:fluxes, :maxiter), Int32(sc.iterations))
        poke!(r, (:fluxes, :tolerance), 0.0)
    else
        poke!(r, (:fluxes, :stop_kind), STOP_CONVERGENCE)
        poke!(r, (:fluxes, :maxiter), Int32(sc.maxiter))
        poke!(r, (:fluxes, :tolerance), sc.tolerance)
    end
end
pack_fluxes!(r, f) = throw(Unsupported(f))

# InterfaceProperties (interface_states.jl:8-12, 20-90, 284-360, 371-391)
function pack_interface_properties!(r, props)
    q = props.specific_humidity_formulation
    q isa IC.ImpureSaturationSpecificHumidity || throw(Unsupported(q))
    poke!(r, (:humidity_phase,), nameof(typeof(q.phase)) === :Ice ? PHASE_ICE : PHASE_LIQUID)
    x = q.water_mole_fraction
    x isa Union{Nothing, Number} || throw(Unsupported(x))
    poke!(r, (:has_water_mole_fraction,), Int32(isnothing(x) ? 0 : 1))
    poke!(r, (:water_mole_fraction,), isnothing(x) ? 1.0 : x)
    poke!(r, (:velocity_formulation,), props.velocity_formulation isa IC.WindVelocity ? WIND_VELOCITY : RELATIVE_VELOCITY)
    t = props.temperature_formulation
    if t isa IC.SkinTemperature
        poke!(r, (:max_delta_T,), t.max_ΔT)
        flux = t.internal_flux
        name = nameof(typeof(flux))
        if name === :IceSnowConductiveFlux
            poke!(r, (:temperature_formulation,), SKIN_TEMPERATURE_CONDUCTIVE)
            poke!(r, (:ice_conductivity,), flux.ice_conductivity)
            poke!(r, (:snow_conductivity,), flux.snow_conductivity)
        elseif name === :ConductiveFlux
            poke!(r, (:temperature_formulation,), SKIN_TEMPERATURE_CONDUCTIVE)
            poke!(r, (:ice_conductivity,), flux.conductivity)
            poke!(r, (:snow_conductivity,), 0.0)
        elseif flux isa IC.DiffusiveFlux
            poke!(r, (:temperature_formulation,), SKIN_TEMPERATURE_DIFFUSIVE)
            κ = flux.κ
            poke!(r, (:diffusive_kappa,), κ isa IC.InteriorDiffusivity ? κ.minimum_diffusivity : κ)
            poke!(r, (:diffusive_delta,), flux.δ)
        else
            throw(Unsupported(flux))
        end
    else
        t isa IC.BulkTemperature || throw(Unsupported(t))
        poke!(r, (:temperature_formulation,), BULK_TEMPERATURE)
    end
end

celsius_offset(units) = nameof(typeof(units)) === :DegreesCelsius ? 273.15 : 0.0

# The parameters of one atmosphere interface of `model` (`which`: :ocean or :sea_ice).
function interface_params(model, interface, which)
    r = Ref{InterfaceParams}()
    if which === :ocean
        ccall((:nesf_default_ao_params, libnesf), Cvoid, (Ref{InterfaceParams},), r)
    else
        ccall((:nesf_default_ai_params, libnesf), Cvoid, (Ref{InterfaceParams},), r)
    end
    pack_fluxes!(r, unwrap(interface.flux_formulation))
    pack_thermodynamics!(r, thermodynamics_parameters(model.atmosphere))
    pack_interface_properties!(r, interface.properties)
    props = model.interfaces.properties
    poke!(r, (:gravitational_acceleration,), props.gravitational_acceleration)
    poke!(r, (:surface_layer_height,), props.surface_layer_height)
    poke!(r, (:boundary_layer_height,), boundary_layer_height(model.atmosphere))
    ocean = model.interfaces.ocean_properties
    poke!(r, (:interior_temperature_offset,), celsius_offset(ocean.temperature_units))
    poke!(r, (:interface_temperature_offset,),
          which === :ocean ? celsius_offset(ocean.temperature_units) :
                             celsius_offset(model.interfaces.sea_ice_properties.temperature_units))
    poke!(r, (:interior_reference_density,), ocean.reference_density)
    poke!(r, (:interior_heat_capacity,), ocean.heat_capacity)
    if which === :sea_ice
        liq = model.sea_ice.model.phase_transitions.liquidus
        poke!(r, (:liquidus_freshwater_melting_temperature,), liq.freshwater_melting_temperature)
        poke!(r, (:liquidus_slope,), liq.slope)
    end
    rad = model.radiation
    # the surface's radiation properties (air_sea_interface_radiation_state.jl:30-38): none
    # means no interface radiative forcing
    surf = isnothing(rad) ? nothing : get(rad.surface_properties, which === :ocean ? :ocean : :sea_ice, nothing)
    if isnothing(surf)
        poke!(r, (:has_radiation,), Int32(0))
    else
        (surf.albedo isa Number && surf.emissivity isa Number) || throw(Unsupported(surf))
        poke!(r, (:has_radiation,), Int32(1))
        poke!(r, (:stefan_boltzmann_constant,), rad.stefan_boltzmann_constant)
        poke!(r, (:albedo,), surf.albedo)
        poke!(r, (:emissivity,), surf.emissivity)
    end
    return r
end

# Falls back to the reference's generic method when the library does not implement a
# formulation (the packers throw Unsupported).
macro or_reference(call, fallback)
    quote
        try
            $(esc(call))
        catch err
            err isa Unsupported || rethrow()
            $(esc(fallback))
        end
    end
end

# ------------------------------------------------ update_state! phase 2: fluxes
# compute_atmosphere_ocean_fluxes!(coupled_model) (atmosphere_ocean_fluxes.jl:17-60)
function IC.compute_atmosphere_ocean_fluxes!(model::GB300Model)
    @or_reference(ao_fluxes!(model), invoke(IC.compute_atmosphere_ocean_fluxes!, Tuple{Any}, model))
    return nothing
end

function ao_fluxes!(model)
    exchanger = model.interfaces.exchanger
    grid = exchanger.grid
    interface = model.interfaces.atmosphere_ocean_interface
    params = interface_params(model, interface, :ocean)
    atmos, ocean, out = exchanger.atmosphere.state, exchanger.ocean.state, interface.fluxes
    rad = isnothing(exchanger.radiation) ? nothing : exchanger.radiation.state
    kN = size(parent(ocean.T), 3)   # the surface level of the parent array (k = Nz + Hz)
    fields = AOFields(grid_struct(grid), dtype_of(grid), 0,
                      devptr(atmos.u), devptr(atmos.v), devptr(atmos.T), devptr(atmos.p), devptr(atmos.q),
                      surface_ptr(ocean.u, kN), surface_ptr(ocean.v, kN), surface_ptr(ocean.T, kN),
                      surface_ptr(ocean.S, kN), C_NULL,
                      isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˢʷ), isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˡʷ), C_NULL,
                      devptr(out.latent_heat), devptr(out.sensible_heat), devptr(out.water_vapor),
                      devptr(out.x_momentum), devptr(out.y_momentum),
                      devptr(out.friction_velocity), devptr(out.temperature_scale), devptr(out.water_vapor_scale),
                      devptr(interface.temperature), C_NULL)
    check(ccall((:nesf_compute_atmosphere_ocean_fluxes, libnesf), Cint,
                (Ptr{Cvoid}, Ref{InterfaceParams}, Ref{AOFields}, Ref{SolverOptions}, Ptr{Cvoid}, Ptr{Cvoid}),
                C_NULL, params, fields, solver_options(model), C_NULL, stream()))
end

# compute_atmosphere_sea_ice_fluxes!(coupled_model) (atmosphere_sea_ice_fluxes.jl:18-62)
function IC.compute_atmosphere_sea_ice_fluxes!(model::GB300Model)
    isnothing(model.interfaces.atmosphere_sea_ice_interface) && return nothing
    @or_reference(ai_fluxes!(model), invoke(IC.compute_atmosphere_sea_ice_fluxes!, Tuple{Any}, model))
    return nothing
end

function ai_fluxes!(model)
    exchanger = model.interfaces.exchanger
    grid = exchanger.grid
    interface = model.interfaces.atmosphere_sea_ice_interface
    params = interface_params(model, interface, :sea_ice)
    atmos, ice, ocean, out = exchanger.atmosphere.state, exchanger.sea_ice.state, exchanger.ocean.state, interface.fluxes
    rad = isnothing(exchanger.radiation) ? nothing : exchanger.radiation.state
    fields = AIFields(grid_struct(grid), dtype_of(grid), 0,
                      devptr(atmos.u), devptr(atmos.v), devptr(atmos.T), devptr(atmos.p), devptr(atmos.q),
                      devptr(ocean.T), devptr(ocean.S),
                      devptr(ice.hi), ice.hs isa Oceananigans.Fields.ZeroField ? C_NULL : devptr(ice.hs), devptr(ice.hc),
                      devptr(ice.ℵ), C_NULL,
                      isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˢʷ), isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˡʷ),
                      devptr(interface.temperature),
                      devptr(out.latent_heat), devptr(out.sensible_heat), devptr(out.water_vapor),
                      devptr(out.x_momentum), devptr(out.y_momentum), C_NULL)
    check(ccall((:nesf_compute_atmosphere_sea_ice_fluxes, libnesf), Cint,
                (Ptr{Cvoid}, Ref{InterfaceParams}, Ref{AIFields}, Ref{SolverOptions}, Ptr{Cvoid}, Ptr{Cvoid}),
                C_NULL, params, fields, solver_options(model), C_NULL, stream()))
end

# compute_sea_ice_ocean_fluxes!(coupled_model) (sea_ice_ocean_fluxes.jl:20-77): the frazil
# column over the ocean's levels, the interface heat, salt and freshwater fluxes. The
# ice-ocean stress (a sea-ice dynamics kernel, sea_ice_ocean_fluxes.jl:79-104) stays with
# the reference.
function IC.compute_sea_ice_ocean_fluxes!(model::GB300Model)
    interface = model.interfaces.sea_ice_ocean_interface
    isnothing(interface) && return nothing
    @or_reference(io_fluxes!(model, interface), invoke(IC.compute_sea_ice_ocean_fluxes!, Tuple{Any}, model))
    return nothing
end

function io_params(model, interface)
    f = interface.flux_formulation
    sea_ice = model.sea_ice
    ocean = model.interfaces.ocean_properties
    pt = sea_ice.model.phase_transitions
    T = ESM.ocean_temperature(model.ocean)
    name = nameof(typeof(f))
    p = Ref{IOParams}()
    ccall((:nesf_default_io_params, libnesf), Cvoid, (Ref{IOParams},), p)
    if name === :IceBathHeatFlux
        poke!(p, (:formulation,), Int32(1))
        poke!(p, (:conductive,), Int32(0))
        poke!(p, (:heat_transfer_coefficient,), f.heat_transfer_coefficient)
        poke!(p, (:friction_velocity,), f.friction_velocity)
    elseif name === :ThreeEquationHeatFlux
        poke!(p, (:formulation,), Int32(0))
        conductive = nameof(typeof(f.internal_heat_flux)) === :ConductiveFlux
        poke!(p, (:conductive,), Int32(conductive ? 1 : 0))
        poke!(p, (:heat_transfer_coefficient,), f.heat_transfer_coefficient)
        poke!(p, (:salt_transfer_coefficient,), f.salt_transfer_coefficient)
        f.friction_velocity isa Number || throw(Unsupported(f.friction_velocity))
        poke!(p, (:friction_velocity,), f.friction_velocity)
        conductive && poke!(p, (:ice_conductivity,), f.internal_heat_flux.conductivity)
    else
        throw(Unsupported(f))
    end
    poke!(p, (:reference_latent_heat,), pt.reference_latent_heat)
    poke!(p, (:liquidus_freshwater_melting_temperature,), pt.liquidus.freshwater_melting_temperature)
    poke!(p, (:liquidus_slope,), pt.liquidus.slope)
    poke!(p, (:ocean_reference_density,), ocean.reference_density)
    poke!(p, (:ocean_heat_capacity,), ocean.heat_capacity)
    poke!(p, (:dt,), sea_ice.Δt)
    Nx, Ny, Nz = size(T.grid)
    Hx, Hy, _ = halo_size(T.grid)
    poke!(p, (:nz,), Int32(Nz))
    poke!(p, (:stride_k,), Int64((Nx + 2Hx) * (Ny + 2Hy)))
    return p
end

function io_fluxes!(model, interface)
    sea_ice = model.sea_ice
    grid = sea_ice.model.grid
    T, S = ESM.ocean_temperature(model.ocean), ESM.ocean_salinity(model.ocean)
    _, _, Hz = halo_size(T.grid)
    Δz = CuArray([Oceananigans.Operators.Δzᶜᶜᶜ(1, 1, k, T.grid) for k in 1:size(T.grid, 3)])
    out = interface.fluxes
    mf = sea_ice.model.mass_fluxes.thermodynamics
    params = io_params(model, interface)
    fields = IOFields(grid_struct(grid), dtype_of(grid), 0,
                      surface_ptr(T, Hz + 1), surface_ptr(S, Hz + 1), reinterpret(Ptr{Float64}, pointer(Δz)),
                      devptr(sea_ice.model.tracers.S), devptr(sea_ice.model.ice_thickness),
                      devptr(sea_ice.model.ice_consolidation_thickness), devptr(sea_ice.model.ice_concentration),
                      devptr(interface.temperature), devptr(mf.ice), devptr(mf.snow),
                      devptr(out.interface_heat), devptr(out.frazil_heat), devptr(out.salt), devptr(out.freshwater),
                      devptr(interface.temperature), devptr(interface.salinity))
    GC.@preserve Δz check(ccall((:nesf_compute_sea_ice_ocean_fluxes, libnesf), Cint,
                                (Ptr{Cvoid}, Ref{IOParams}, Ref{IOFields}, Ptr{Cvoid}),
                                C_NULL, params, fields, stream()))
end

# ----------------------------------------------- update_state! phase 1: the atmosphere
# interpolate_state!(exchanger, grid, ::PrescribedAtmosphere, coupled_model)
# (interpolate_atmospheric_state.jl:9-137) on a regular longitude-latitude exchange grid,
# whose fractional indices the library computes per tile from the coordinates. The
# snapshot pair is n1, n2 of the FieldTimeSeries (cpu_interpolating_time_indices
# restated by nesf_time_indices); stride_t is the distance between their slots. The
# barotropic potential forcing and other exchange grids stay with the reference.
function ESM.interpolate_state!(exchanger, grid::LatitudeLongitudeGrid, atmosphere::PrescribedAtmosphere,
                                model::GB300Model)
    @or_reference(interpolate_atmosphere!(exchanger, grid, atmosphere, model),
                  invoke(ESM.interpolate_state!, Tuple{Any, Any, PrescribedAtmosphere, Any},
                         exchanger, grid, atmosphere, model))
    return nothing
end

function time_pair(u::FieldTimeSeries, t)
    times = collect(Float64, u.times)
    indexing = nameof(typeof(u.time_indexing))
    code = indexing === :Cyclical ? Int32(0) : indexing === :Linear ? Int32(1) : indexing === :Clamp ? Int32(2) :
           throw(Unsupported(u.time_indexing))
    period = indexing === :Cyclical ? Float64(u.time_indexing.period) : 0.0
    n1, n2, w = Ref{Int32}(), Ref{Int32}(), Ref{Float64}()
    check(ccall((:nesf_time_indices, libnesf), Cint,
                (Ptr{Float64}, Int32, Int32, Float64, Float64, Ref{Int32}, Ref{Int32}, Ref{Float64}),
                times, length(times), code, period, Float64(t), n1, n2, w))
    nameof(typeof(u.backend)) === :InMemory && u.backend.length === nothing || throw(Unsupported(u.backend))
    return n1[] + 1, n2[] + 1, w[]
end

function interpolate_atmosphere!(exchanger, grid, atmosphere, model)
    ua = atmosphere.velocities.u
    n1, n2, w = time_pair(ua, model.clock.time)
    ag = atmosphere.grid
    ag isa LatitudeLongitudeGrid || throw(Unsupported(ag))
    Nxa, Nya, _ = size(ag)
    Hxa, Hya, _ = halo_size(ag)
    plane = (Nxa + 2Hxa) * (Nya + 2Hya)
    λa, φa = ag.λᶜᵃᵃ, ag.φᵃᶜᵃ
    λ, φ = grid.λᶜᵃᵃ, grid.φᵃᶜᵃ
    atmos = AtmosGrid(Nxa, Nya, Hxa, Hya, Nxa + 2Hxa, (n2 - n1) * plane,
                      λa[1], λa[2] - λa[1], φa[1], φa[2] - φa[1])
    coords = ExchangeCoords(λ[1], λ[2] - λ[1], φ[1], φ[2] - φ[1])
    snap(fts) = isnothing(fts) ? C_NULL : reinterpret(Ptr{Cvoid}, pointer(view(parent(fts.data), :, :, 1, n1)))
    rain, snow = atmosphere.precipitation_flux.rain, atmosphere.precipitation_flux.snow
    st = exchanger.state
    fields = InterpFields(grid_struct(grid), coords, atmos, dtype_of(grid), 0, w,
                          snap(atmosphere.velocities.u), snap(atmosphere.velocities.v), snap(atmosphere.temperature),
                          snap(atmosphere.specific_humidity), snap(atmosphere.pressure), snap(rain), snap(snow),
                          C_NULL, C_NULL,
                          devptr(st.u), devptr(st.v), devptr(st.T), devptr(st.q), devptr(st.p),
                          devptr(st.Jʳⁿ), devptr(st.Jˢⁿ), C_NULL, C_NULL, C_NULL, C_NULL)
    check(ccall((:nesf_interpolate_atmosphere_state, libnesf), Cint, (Ref{InterpFields}, Ptr{Cvoid}),
                fields, stream()))
end

# --------------------------------------------- update_state! phases 3 and 4: assembly
# The assembly of the net ocean and sea-ice fluxes (assemble_net_ocean_fluxes.jl:16-153,
# assemble_net_sea_ice_fluxes.jl:11-81) and the radiative add-ons
# (apply_air_sea_radiative_fluxes.jl:18-111, apply_air_sea_ice_radiative_fluxes.jl:15-90),
# one argument bundle for all four.
function assembly_params(model)
    ocean = model.interfaces.ocean_properties
    p = Ref{AssemblyParams}()
    ccall((:nesf_default_assembly_params, libnesf), Cvoid, (Ref{AssemblyParams},), p)
    poke!(p, (:ocean_reference_density,), ocean.reference_density)
    poke!(p, (:ocean_heat_capacity,), ocean.heat_capacity)
    poke!(p, (:interface_temperature_offset,), celsius_offset(ocean.temperature_units))
    rad = model.radiation
    if !isnothing(rad)
        so, si = get(rad.surface_properties, :ocean, nothing), get(rad.surface_properties, :sea_ice, nothing)
        (!isnothing(so) && !isnothing(si) && so.albedo isa Number && si.albedo isa Number) ||
            throw(Unsupported(rad.surface_properties))
        poke!(p, (:stefan_boltzmann_constant,), rad.stefan_boltzmann_constant)
        poke!(p, (:ocean_albedo,), so.albedo)
        poke!(p, (:ocean_emissivity,), so.emissivity)
        poke!(p, (:ice_albedo,), si.albedo)
        poke!(p, (:ice_emissivity,), si.emissivity)
    end
    return p
end

function assembly_fields(model)
    ifc = model.interfaces
    ex = ifc.exchanger
    grid = ex.grid
    atmos = ex.atmosphere.state
    ao, ai, io = ifc.atmosphere_ocean_interface, ifc.atmosphere_sea_ice_interface, ifc.sea_ice_ocean_interface
    net, ice_net = ifc.net_fluxes.ocean, isnothing(ai) ? nothing : ifc.net_fluxes.sea_ice
    rad = isnothing(ex.radiation) ? nothing : ex.radiation.state
    rf = isnothing(model.radiation) ? nothing : model.radiation.interface_fluxes
    ocean_diag = isnothing(rf) || !haskey(rf, :ocean) ? nothing : rf.ocean
    ice_diag = isnothing(rf) || !haskey(rf, :sea_ice) ? nothing : rf.sea_ice
    T = ESM.ocean_temperature(model.ocean)
    kN = size(parent(T), 3)
    aleph = isnothing(model.sea_ice) ? nothing : ESM.sea_ice_concentration(model.sea_ice)
    d(x) = isnothing(x) ? C_NULL : devptr(x)
    g(nt, name) = isnothing(nt) ? C_NULL : devptr(getproperty(nt, name))
    return AssemblyFields(grid_struct(grid), dtype_of(grid), 0,
        C_NULL, d(aleph), surface_ptr(T, kN), devptr(atmos.Jʳⁿ), devptr(atmos.Jˢⁿ), C_NULL, C_NULL,
        devptr(ao.fluxes.sensible_heat), devptr(ao.fluxes.latent_heat), devptr(ao.fluxes.water_vapor),
        devptr(ao.fluxes.x_momentum), devptr(ao.fluxes.y_momentum), devptr(ao.temperature),
        g(isnothing(io) ? nothing : io.fluxes, :interface_heat), g(isnothing(io) ? nothing : io.fluxes, :frazil_heat),
        g(isnothing(io) ? nothing : io.fluxes, :salt), g(isnothing(io) ? nothing : io.fluxes, :freshwater),
        g(isnothing(io) ? nothing : io.fluxes, :x_momentum), g(isnothing(io) ? nothing : io.fluxes, :y_momentum),
        g(isnothing(ai) ? nothing : ai.fluxes, :sensible_heat), g(isnothing(ai) ? nothing : ai.fluxes, :latent_heat),
        g(isnothing(ai) ? nothing : ai.fluxes, :x_momentum), g(isnothing(ai) ? nothing : ai.fluxes, :y_momentum),
        isnothing(ai) ? C_NULL : devptr(ai.temperature),
        isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˢʷ), isnothing(rad) ? C_NULL : devptr(rad.ℐꜜˡʷ),
        devptr(net.u), devptr(net.v), devptr(net.T), devptr(net.S), devptr(net.η), devptr(net.freshwater_heat_content),
        isnothing(ice_net) ? C_NULL : devptr(ice_net.top.heat), isnothing(ice_net) ? C_NULL : devptr(ice_net.top.snowfall),
        isnothing(ice_net) ? C_NULL : devptr(ice_net.top.u), isnothing(ice_net) ? C_NULL : devptr(ice_net.top.v),
        isnothing(ice_net) ? C_NULL : devptr(ice_net.bottom.heat),
        g(ocean_diag, :upwelling_longwave), g(ocean_diag, :downwelling_longwave), g(ocean_diag, :downwelling_shortwave),
        g(ice_diag, :upwelling_longwave), g(ice_diag, :downwelling_longwave), g(ice_diag, :downwelling_shortwave))
end

function run_assembly!(model, entry::Symbol)
    params = assembly_params(model)
    fields = assembly_fields(model)
    check(ccall((entry, libnesf), Cint, (Ref{AssemblyParams}, Ref{AssemblyFields}, Ptr{Cvoid}),
                params, fields, stream()))
end

ESM.update_net_fluxes!(model::GB300Model, ocean::NumericalEarth.Oceans.OceananigansModelSimulations) =
    @or_reference(run_assembly!(model, :nesf_assemble_net_ocean_fluxes),
                  invoke(ESM.update_net_fluxes!, Tuple{Any, NumericalEarth.Oceans.OceananigansModelSimulations},
                         model, ocean))

ESM.update_net_fluxes!(model::GB300Model, sea_ice::Simulation{<:SeaIceModel}) =
    @or_reference(run_assembly!(model, :nesf_assemble_net_sea_ice_fluxes),
                  invoke(ESM.update_net_fluxes!, Tuple{Any, Simulation{<:SeaIceModel}}, model, sea_ice))

function ESM.apply_air_sea_radiative_fluxes!(model::GB300Model)
    (isnothing(model.radiation) || isnothing(model.ocean)) && return nothing
    @or_reference(run_assembly!(model, :nesf_apply_air_sea_radiative_fluxes),
                  invoke(ESM.apply_air_sea_radiative_fluxes!, Tuple{EarthSystemModel}, model))
    return nothing
end

function ESM.apply_air_sea_ice_radiative_fluxes!(model::GB300Model)
    (isnothing(model.radiation) || !(model.sea_ice isa Simulation{<:SeaIceModel})) && return nothing
    @or_reference(run_assembly!(model, :nesf_apply_air_sea_ice_radiative_fluxes),
                  invoke(ESM.apply_air_sea_ice_radiative_fluxes!, Tuple{EarthSystemModel}, model))
    return nothing
end

# ------------------------------------------------------ the land interface
# compute_atmosphere_land_fluxes!(coupled_model, interface) (atmosphere_land_fluxes.jl:48-110)
# for an atmosphere-land interface built with
#     atmosphere_land_interface(grid, atmosphere, land;
#                               fluxes = NESF.GB300SimilarityTheoryFluxes(default_atmosphere_land_fluxes(land)))
# the wrapped formulation packed as for the ocean, the humidity model the interface's own.
const HUMIDITY = (impure = Int32(0), bulk = Int32(1), fractional = Int32(2), skin = Int32(3), dry_layer = Int32(4))

humidity_params!(r, q) = throw(Unsupported(q))
humidity_params!(r, ::IC.ImpureSaturationSpecificHumidity) = poke!(r, (:humidity_formulation,), HUMIDITY.impure)
function humidity_params!(r, ::IC.BulkHumidity)
    poke!(r, (:humidity_formulation,), HUMIDITY.bulk)
    poke!(r, (:evaporation_efficiency,), 1.0)
end
function humidity_params!(r, q::IC.FractionalHumidity)
    poke!(r, (:humidity_formulation,), HUMIDITY.fractional)
    if q.efficiency isa IC.CriticalSaturation
        poke!(r, (:critical_saturation,), q.efficiency.critical_saturation)
    else
        poke!(r, (:critical_saturation,), 0.0)
        poke!(r, (:evaporation_efficiency,), q.efficiency)
    end
end
function humidity_params!(r, q::IC.SkinHumidity)
    poke!(r, (:humidity_formulation,), HUMIDITY.skin)
    poke!(r, (:skin_surface_thickness,), q.surface_thickness)
    poke!(r, (:skin_vapor_diffusivity,), q.vapor_diffusivity)
end
function humidity_params!(r, q::IC.DryLayerHumidity)
    d, v = q.dry_layer_depth, q.vapor_exchange
    poke!(r, (:humidity_formulation,), HUMIDITY.dry_layer)
    poke!(r, (:tortuosity,), Int32(v.tortuosity isa IC.PowerLawTortuosity ? 1 : 0))
    poke!(r, (:maximum_dry_layer_depth,), d.maximum_dry_layer_depth)
    poke!(r, (:dry_layer_onset_saturation,), d.dry_layer_onset_saturation)
    poke!(r, (:dry_layer_exponent,), d.dry_layer_exponent)
    poke!(r, (:minimum_dry_layer_depth,), v.minimum_dry_layer_depth)
    poke!(r, (:molecular_diffusivity,), v.molecular_diffusivity)
    poke!(r, (:wet_transition_width,), v.wet_transition_width)
    poke!(r, (:thermal_exchange_depth,), q.thermal_exchange_depth)
    poke!(r, (:porosity,), q.porosity)
end

function IC.compute_atmosphere_land_fluxes!(model, interface::IC.AtmosphereInterface{<:Any, <:GB300SimilarityTheoryFluxes})
    @or_reference(al_fluxes!(model, interface),
                  invoke(IC.compute_atmosphere_land_fluxes!, Tuple{Any, IC.AtmosphereInterface}, model, interface))
    return nothing
end

function al_fluxes!(model, interface)
    exchanger = model.interfaces.exchanger
    grid = exchanger.grid
    atmos, land, out = exchanger.atmosphere.state, exchanger.land.state, interface.fluxes
    r = Ref{InterfaceParams}()
    ccall((:nesf_default_al_params, libnesf), Cvoid, (Ref{InterfaceParams},), r)
    pack_fluxes!(r, unwrap(interface.flux_formulation))
    pack_thermodynamics!(r, thermodynamics_parameters(model.atmosphere))
    humidity_params!(r, interface.properties.specific_humidity_formulation)
    poke!(r, (:velocity_formulation,),
          interface.properties.velocity_formulation isa IC.WindVelocity ? WIND_VELOCITY : RELATIVE_VELOCITY)
    props = model.interfaces.properties
    poke!(r, (:gravitational_acceleration,), props.gravitational_acceleration)
    poke!(r, (:surface_layer_height,), props.surface_layer_height)
    poke!(r, (:boundary_layer_height,), boundary_layer_height(model.atmosphere))
    fields = ALFields(grid_struct(grid), dtype_of(grid), 0,
                      devptr(atmos.u), devptr(atmos.v), devptr(atmos.T), devptr(atmos.p), devptr(atmos.q),
                      devptr(land.T), devptr(land.saturation),
                      devptr(out.latent_heat), devptr(out.sensible_heat), devptr(out.water_vapor),
                      devptr(out.x_momentum), devptr(out.y_momentum),
                      devptr(out.friction_velocity), devptr(out.temperature_scale), devptr(out.water_vapor_scale),
                      devptr(interface.temperature), C_NULL)
    opts = SolverOptions(precision_code(interface.flux_formulation), 0, 0, 0, 0, 0, C_NULL, 10.0, 2e-6, 0.9, 0.7)
    check(ccall((:nesf_compute_atmosphere_land_fluxes, libnesf), Cint,
                (Ptr{Cvoid}, Ref{InterfaceParams}, Ref{ALFields}, Ref{SolverOptions}, Ptr{Cvoid}, Ptr{Cvoid}),
                C_NULL, r, fields, opts, C_NULL, stream()))
end

end # module
