# NESF.jl -- ccall shim that routes NumericalEarth.jl's interface-flux step to
# libnesf.so. Not executed in this repository (no Julia toolchain here); it is the
# binding a NumericalEarth maintainer would add, written against include/nesf.h.
#
# Usage:
#     using NumericalEarth, NESF
#     fluxes = NESF.GB300SimilarityTheoryFluxes(SimilarityTheoryFluxes(); precision = :f32)
#     interfaces = ComponentInterfaces(atmosphere, ocean, sea_ice; atmosphere_ocean_fluxes = fluxes)
#
# The methods below specialise compute_atmosphere_ocean_fluxes! on models whose
# atmosphere-ocean flux formulation is the wrapper (and compute_atmosphere_land_fluxes! on
# an atmosphere-land interface built with it), and call the library with the device
# pointers of the Oceananigans fields (parent arrays, halo included).
module NESF

using CUDA
using Oceananigans: Oceananigans, architecture, size, halo_size
using NumericalEarth.EarthSystemModels.InterfaceComputations: InterfaceComputations
const IC = InterfaceComputations

const libnesf = get(ENV, "NESF_LIB", joinpath(@__DIR__, "..", "nesf", "libnesf.so"))

const NESF_OK = Cint(0)
const NESF_F64 = Int32(0)
const NESF_F32 = Int32(1)
const NESF_PLAIN_F64 = Int32(0)
const NESF_F32_POLISH = Int32(1)
const NESF_F32_ADAPTIVE = Int32(2)

struct Grid
    nx::Int32; ny::Int32; hx::Int32; hy::Int32; stride_j::Int64
end

# Opaque blob holding nesf_interface_params, filled by the library defaults
# and then patched field by field through the offsets exported by the library's
# layout (the Python binding nesf/_abi.py lists the field order).
const PARAMS_BYTES = 1536   # sizeof(nesf_interface_params); nesf_struct_sizes() reports it

struct AOFields
    grid::Grid; dtype::Int32; pad::Int32
    u_atm::Ptr{Cvoid}; v_atm::Ptr{Cvoid}; T_atm::Ptr{Cvoid}; p_atm::Ptr{Cvoid}; q_atm::Ptr{Cvoid}
    u_oc::Ptr{Cvoid}; v_oc::Ptr{Cvoid}; T_oc::Ptr{Cvoid}; S_oc::Ptr{Cvoid}; inactive::Ptr{UInt8}
    sw_down::Ptr{Cvoid}; lw_down::Ptr{Cvoid}; kappa::Ptr{Cvoid}
    latent_heat::Ptr{Cvoid}; sensible_heat::Ptr{Cvoid}; water_vapor::Ptr{Cvoid}
    x_momentum::Ptr{Cvoid}; y_momentum::Ptr{Cvoid}
    friction_velocity::Ptr{Cvoid}; temperature_scale::Ptr{Cvoid}; water_vapor_scale::Ptr{Cvoid}
    interface_temperature::Ptr{Cvoid}; iterations::Ptr{Int32}
end

# nesf_solver_options; block_size, schedule and ctas_per_sm are reserved (the launch shapes are
# the library context's tuning, nesf_set_tuning / nesf_autotune).
struct SolverOptions
    precision::Int32; polish_maxiter::Int32; block_size::Int32; schedule::Int32
    ctas_per_sm::Int32; warm_start::Int32; mlp::Ptr{Cvoid}; fallback_ratio::Float64; path_tolerance::Float64
    fp32_rho::Float64
end

struct GB300SimilarityTheoryFluxes{F}
    inner :: F                  # the reference formulation (defaults, solver settings)
    precision :: Symbol         # :f64 (drop-in), :f32 (FP32 sweep + FP64 Newton polish) or
                   # :f32_adaptive (FP32 result kept where well conditioned)
end
GB300SimilarityTheoryFluxes(inner; precision = :f64) = GB300SimilarityTheoryFluxes(inner, precision)

check(code) = code == NESF_OK ||
    error("nesf error $code: " * unsafe_string(ccall((:nesf_last_error, libnesf), Cstring, ())))

devptr(f) = reinterpret(Ptr{Cvoid}, pointer(parent(f)))   # CuArray parent of an Oceananigans field
surface(f, k) = view(parent(f), :, :, k)                   # k = Nz + Hz slice of a 3-D field

function default_params(interface::Symbol)
    buf = zeros(UInt8, PARAMS_BYTES)
    fn = interface === :ocean ? :nesf_default_ao_params :
         interface === :land ? :nesf_default_al_params : :nesf_default_ai_params
    ccall((fn, libnesf), Cvoid, (Ptr{UInt8},), buf)
    return buf
end

function InterfaceComputations.compute_atmosphere_ocean_fluxes!(coupled_model, fluxes::GB300SimilarityTheoryFluxes)
    exchanger = coupled_model.interfaces.exchanger
    grid = exchanger.grid
    Nx, Ny, Nz = size(grid)
    Hx, Hy, Hz = halo_size(grid)
    atmos = exchanger.atmosphere.state
    ocean = exchanger.ocean.state
    out = coupled_model.interfaces.atmosphere_ocean_interface.fluxes
    Ts = coupled_model.interfaces.atmosphere_ocean_interface.temperature
    FT = eltype(grid)
    g = Grid(Nx, Ny, Hx, Hy, Nx + 2Hx)
    k = Nz + Hz
    fields = AOFields(g, FT == Float64 ? NESF_F64 : NESF_F32, 0,
         devptr(atmos.u), devptr(atmos.v), devptr(atmos.T), devptr(atmos.p), devptr(atmos.q),
         pointer(surface(ocean.u, k)), pointer(surface(ocean.v, k)),
         pointer(surface(ocean.T, k)), pointer(surface(ocean.S, k)), C_NULL,
         C_NULL, C_NULL, C_NULL,
         devptr(out.latent_heat), devptr(out.sensible_heat), devptr(out.water_vapor),
         devptr(out.x_momentum), devptr(out.y_momentum),
         devptr(out.friction_velocity), devptr(out.temperature_scale), devptr(out.water_vapor_scale),
         devptr(Ts), C_NULL)
    params = default_params(:ocean)
    prec = fluxes.precision === :f32 ? NESF_F32_POLISH :
           fluxes.precision === :f32_adaptive ? NESF_F32_ADAPTIVE : NESF_PLAIN_F64
    opts = SolverOptions(prec, 0, 128, 0, 0, 0, C_NULL, 10.0, 2e-6, 0.9)
    stream = CUDA.stream().handle
    check(ccall((:nesf_compute_atmosphere_ocean_fluxes, libnesf), Cint,
                (Ptr{Cvoid}, Ptr{UInt8}, Ref{AOFields}, Ref{SolverOptions}, Ptr{Cvoid}, Ptr{Cvoid}),
                C_NULL, params, fields, opts, C_NULL, stream))
    return nothing
end

# Byte offsets of the land humidity fields in nesf_interface_params (the Python tests check
# them against the library's layout).
const HUMIDITY_OFFSETS = (
    humidity_formulation = 1424,
    evaporation_efficiency = 1432,
    critical_saturation = 1440,
    skin_surface_thickness = 1448,
    skin_vapor_diffusivity = 1456,
    tortuosity = 1464,
    maximum_dry_layer_depth = 1472,
    dry_layer_onset_saturation = 1480,
    dry_layer_exponent = 1488,
    minimum_dry_layer_depth = 1496,
    molecular_diffusivity = 1504,
    wet_transition_width = 1512,
    thermal_exchange_depth = 1520,
    porosity = 1528)

poke!(buf, name, v::T) where {T} = GC.@preserve buf unsafe_store!(Ptr{T}(pointer(buf) + HUMIDITY_OFFSETS[name]), v)

# The interface's specific_humidity_formulation (interface_states.jl:100-230,
# dry_layer_humidity.jl:216-235) written into the parameter blob.
humidity_params!(buf, q) = nothing   # ImpureSaturationSpecificHumidity: the defaults
function humidity_params!(buf, ::IC.BulkHumidity)
    poke!(buf, :humidity_formulation, Int32(1))
    poke!(buf, :evaporation_efficiency, 1.0)
end
function humidity_params!(buf, q::IC.FractionalHumidity)
    poke!(buf, :humidity_formulation, Int32(2))
    if q.efficiency isa IC.CriticalSaturation
        poke!(buf, :critical_saturation, Float64(q.efficiency.critical_saturation))
    else
        poke!(buf, :critical_saturation, 0.0)
        poke!(buf, :evaporation_efficiency, Float64(q.efficiency))
    end
end
function humidity_params!(buf, q::IC.SkinHumidity)
    poke!(buf, :humidity_formulation, Int32(3))
    poke!(buf, :skin_surface_thickness, Float64(q.surface_thickness))
    poke!(buf, :skin_vapor_diffusivity, Float64(q.vapor_diffusivity))
end
function humidity_params!(buf, q::IC.DryLayerHumidity)
    d, v = q.dry_layer_depth, q.vapor_exchange
    poke!(buf, :humidity_formulation, Int32(4))
    poke!(buf, :tortuosity, Int32(v.tortuosity isa IC.PowerLawTortuosity ? 1 : 0))
    poke!(buf, :maximum_dry_layer_depth, Float64(d.maximum_dry_layer_depth))
    poke!(buf, :dry_layer_onset_saturation, Float64(d.dry_layer_onset_saturation))
    poke!(buf, :dry_layer_exponent, Float64(d.dry_layer_exponent))
    poke!(buf, :minimum_dry_layer_depth, Float64(v.minimum_dry_layer_depth))
    poke!(buf, :molecular_diffusivity, Float64(v.molecular_diffusivity))
    poke!(buf, :wet_transition_width, Float64(v.wet_transition_width))
    poke!(buf, :thermal_exchange_depth, Float64(q.thermal_exchange_depth))
    poke!(buf, :porosity, Float64(q.porosity))
end

struct ALFields
    grid::Grid; dtype::Int32; pad::Int32
    u_atm::Ptr{Cvoid}; v_atm::Ptr{Cvoid}; T_atm::Ptr{Cvoid}; p_atm::Ptr{Cvoid}; q_atm::Ptr{Cvoid}
    land_temperature::Ptr{Cvoid}; saturation::Ptr{Cvoid}
    latent_heat::Ptr{Cvoid}; sensible_heat::Ptr{Cvoid}; water_vapor::Ptr{Cvoid}
    x_momentum::Ptr{Cvoid}; y_momentum::Ptr{Cvoid}
    friction_velocity::Ptr{Cvoid}; temperature_scale::Ptr{Cvoid}; water_vapor_scale::Ptr{Cvoid}
    interface_temperature::Ptr{Cvoid}; iterations::Ptr{Int32}
end

# compute_atmosphere_land_fluxes!(coupled_model, interface) (atmosphere_land_fluxes.jl:48-110)
# for an atmosphere-land interface built with
#     atmosphere_land_interface(grid, atmosphere, land;
#                               fluxes = NESF.GB300SimilarityTheoryFluxes(default_atmosphere_land_fluxes(land)))
# The wrapped formulation's coefficients are the library's land defaults
# (nesf_default_al_params); the humidity model is the interface's own.
function IC.compute_atmosphere_land_fluxes!(coupled_model,
                               interface::IC.AtmosphereInterface{<:Any, <:GB300SimilarityTheoryFluxes})
    exchanger = coupled_model.interfaces.exchanger
    grid = exchanger.grid
    Nx, Ny, Nz = size(grid)
    Hx, Hy, Hz = halo_size(grid)
    atmos = exchanger.atmosphere.state
    land = exchanger.land.state
    out = interface.fluxes
    FT = eltype(grid)
    fields = ALFields(Grid(Nx, Ny, Hx, Hy, Nx + 2Hx), FT == Float64 ? NESF_F64 : NESF_F32, 0,
         devptr(atmos.u), devptr(atmos.v), devptr(atmos.T), devptr(atmos.p), devptr(atmos.q),
         devptr(land.T), devptr(land.saturation),
         devptr(out.latent_heat), devptr(out.sensible_heat), devptr(out.water_vapor),
         devptr(out.x_momentum), devptr(out.y_momentum),
         devptr(out.friction_velocity), devptr(out.temperature_scale), devptr(out.water_vapor_scale),
         devptr(interface.temperature), C_NULL)
    params = default_params(:land)
    humidity_params!(params, interface.properties.specific_humidity_formulation)
    fluxes = interface.flux_formulation
    prec = fluxes.precision === :f32 ? NESF_F32_POLISH :
           fluxes.precision === :f32_adaptive ? NESF_F32_ADAPTIVE : NESF_PLAIN_F64
    opts = SolverOptions(prec, 0, 128, 0, 0, 0, C_NULL, 10.0, 2e-6, 0.9)
    check(ccall((:nesf_compute_atmosphere_land_fluxes, libnesf), Cint,
                (Ptr{Cvoid}, Ptr{UInt8}, Ref{ALFields}, Ref{SolverOptions}, Ptr{Cvoid}, Ptr{Cvoid}),
                C_NULL, params, fields, opts, C_NULL, CUDA.stream().handle))
    return nothing
end

end # module
