/*
 * nesf.h -- C ABI of the GB300-native interface-flux library (libnesf.so).
 *
 * The library is a drop-in for the interface-flux step of NumericalEarth.jl's
 * EarthSystemModel: the similarity-theory (Monin-Obukhov) fixed-point solve at
 * the atmosphere-ocean and atmosphere-sea-ice interfaces, the sea-ice-ocean
 * fluxes, the PrescribedAtmosphere space/time interpolation onto the exchange
 * grid, and the assembly of net ocean and sea-ice boundary fluxes.
 *
 * Conventions (mirroring Oceananigans `parent(field)` arrays):
 *   - every 2-D array is column-major with i fastest; element (i, j), with
 *     Oceananigans' 1-based interior index i in [1-hx, nx+hx], j in [1-hy, ny+hy],
 *     lives at  ptr[(i - 1 + hx) + (j - 1 + hy) * stride_j];
 *   - 3-D ocean fields are passed as the pointer of their k = Nz slice, which
 *     has the same 2-D layout (all fields of one grid share halo sizes);
 *   - array pointers are DEVICE pointers (CuArrays / torch CUDA tensors) unless
 *     an entry point says otherwise; the library never frees caller memory;
 *   - all work is enqueued on the caller's stream (`stream`, a cudaStream_t,
 *     NULL = legacy default stream) and returns without synchronising, except
 *     where a `nesf_stats*` is passed (the stats are read back at the end);
 *   - every entry point returns an nesf_status; nesf_last_error() describes
 *     the most recent failure on the calling thread.
 *
 * Reference interfaces replaced (paths inside NumericalEarth.jl v0.6.2):
 *   src/EarthSystemModels/InterfaceComputations/atmosphere_ocean_fluxes.jl:17
 *   src/EarthSystemModels/InterfaceComputations/atmosphere_sea_ice_fluxes.jl:18
 *   src/EarthSystemModels/InterfaceComputations/sea_ice_ocean_fluxes.jl:20
 *   src/Atmospheres/interpolate_atmospheric_state.jl:9
 *   src/Atmospheres/prescribed_atmosphere_regridder.jl:41
 *   src/Radiations/interpolate_radiation_state.jl:4
 *   src/Oceans/assemble_net_ocean_fluxes.jl:16
 *   src/SeaIces/assemble_net_sea_ice_fluxes.jl:11
 *   src/Radiations/apply_air_sea_radiative_fluxes.jl:18
 *   src/Radiations/apply_air_sea_ice_radiative_fluxes.jl:15
 *   src/EarthSystemModels/time_step_earth_system_model.jl:38 (update_state!)
 */
#ifndef NESF_H
#define NESF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NESF_ABI_VERSION 1

/* ------------------------------------------------------------------ status */
typedef enum {
    NESF_OK = 0,
    NESF_ERR_ARG = 1,          /* bad argument (null pointer, size, kind)        */
    NESF_ERR_NONFINITE = 2,    /* non-finite input detected by the input scan    */
    NESF_ERR_TIMEOUT = 3,      /* a bounded device-side wait gave up             */
    NESF_ERR_CUDA = 4,         /* CUDA runtime error                             */
    NESF_ERR_UNSUPPORTED = 5,  /* option combination not implemented             */
    NESF_ERR_CAPACITY = 6      /* size beyond a fixed capacity                   */
} nesf_status;

typedef enum { NESF_F64 = 0, NESF_F32 = 1 } nesf_dtype;

/* ------------------------------------------------------------------ grid */
typedef struct {
    int32_t nx, ny;        /* interior cells                                   */
    int32_t hx, hy;        /* halo widths of every 2-D array of the call       */
    int64_t stride_j;      /* elements between (i, j) and (i, j+1); >= nx+2hx  */
} nesf_grid;

/* ------------------------------------------------- thermodynamic parameters
 * AtmosphereThermodynamicsParameters, src/Atmospheres/thermodynamic_parameters.jl:61-69,106-116,149-165 */
typedef struct {
    double gas_constant;                     /* R   = 8.3144598  */
    double dry_air_molar_mass;               /* Md  = 0.02897    */
    double water_molar_mass;                 /* Mv  = 0.018015   */
    double dry_air_adiabatic_exponent;       /* kd  = 2/7        */
    double water_vapor_heat_capacity;        /* cpv = 1859       */
    double liquid_water_heat_capacity;       /* cpl = 4181       */
    double water_ice_heat_capacity;          /* cpi = 2100       */
    double reference_vaporization_enthalpy;  /* Lv0 = 2500800    */
    double reference_sublimation_enthalpy;   /* Ls0 = 2834400    */
    double reference_temperature;            /* T0  = 273.16     */
    double triple_point_temperature;         /* Ttr = 273.16     */
    double triple_point_pressure;            /* ptr = 611.657    */
} nesf_thermodynamics_parameters;

/* ----------------------------------------------------- stability functions
 * similarity_theory_turbulent_fluxes.jl:487-532 (Edson momentum), 571-618
 * (Edson scalar), 637-677 (SHEBA), 683-710 (Paulson), 712-725 (Split),
 * 742-752 (linear stable). Coefficients are stored in the field order of the
 * reference struct(s). */
typedef enum {
    NESF_PSI_ZERO = 0,                    /* psi == 0 (neutral)                          */
    NESF_PSI_EDSON_MOMENTUM = 1,          /* c = zmax A+ B+ C+ D+ A- B- C- D- E- F-     */
    NESF_PSI_EDSON_SCALAR = 2,            /* c = zmax A+ B+ C+ D+ E+ A- B- C- D- E- F-  */
    NESF_PSI_SHEBA_PAULSON_MOMENTUM = 3,  /* c = sheba a b, paulson a b                  */
    NESF_PSI_SHEBA_PAULSON_SCALAR = 4,    /* c = sheba a b c, paulson a                  */
    NESF_PSI_LINEAR_PAULSON_MOMENTUM = 5, /* c = linear coef zmax, paulson a b           */
    NESF_PSI_LINEAR_PAULSON_SCALAR = 6    /* c = linear coef zmax, paulson a             */
} nesf_psi_kind;

typedef struct {
    int32_t kind;
    int32_t pad_;
    double c[12];
} nesf_stability_function;

/* -------------------------------------------------------- roughness lengths
 * roughness_lengths.jl:1-16 (structs), 74-75 (gravity wave parameter), 93-139
 * (constructors), 182-189 (viscosity), 197-246 (roughness_length). */
typedef enum {
    NESF_ROUGHNESS_CONSTANT = 0,  /* a Number: ell = value                     */
    NESF_ROUGHNESS_MOMENTUM = 1,  /* MomentumRoughnessLength                   */
    NESF_ROUGHNESS_SCALAR = 2     /* ScalarRoughnessLength + ReynoldsScaling    */
} nesf_roughness_kind;

typedef struct {
    int32_t kind;
    int32_t wave_kind;            /* 0: constant Charnock; 1: WindDependentWaveFormulation */
    int32_t viscosity_kind;       /* 0: constant nu; 1: TemperatureDependentAirViscosity   */
    int32_t pad_;
    double value;                 /* constant length                                       */
    double gravitational_acceleration;
    double air_kinematic_viscosity;       /* nu (constant)                                 */
    double viscosity_coefficients[4];     /* C0..C3 of the temperature-dependent law       */
    double charnock;                      /* constant wave_formulation (0.02)              */
    double wave_umax, wave_c1, wave_c2;   /* WindDependentWaveFormulation(Umax, C1, C2)    */
    double smooth_wall_parameter;         /* 0.11                                          */
    double maximum_roughness_length;
    double reynolds_A, reynolds_b;        /* ReynoldsScalingFunction(A, b)                 */
} nesf_roughness_length;

/* --------------------------------------------------- SimilarityTheoryFluxes
 * similarity_theory_turbulent_fluxes.jl:9-18,174-214; compute_interface_state.jl:5-24 */
typedef enum { NESF_SUBGRID_NONE = 0, NESF_SUBGRID_CONSTANT = 1, NESF_SUBGRID_CONVECTIVE = 2 } nesf_subgrid_kind;
typedef enum { NESF_STOP_CONVERGENCE = 0, NESF_STOP_FIXED_ITERATIONS = 1 } nesf_stop_kind;
typedef enum { NESF_PROFILE_LOGARITHMIC = 0, NESF_PROFILE_COARE = 1 } nesf_profile_kind;

typedef struct {
    double von_karman_constant;          /* 0.4  */
    double turbulent_prandtl_number;     /* 1    */
    int32_t subgrid_kind;                /* convective part of SubgridVelocityCorrection       */
    int32_t similarity_form;             /* nesf_profile_kind                                  */
    double gustiness_parameter;          /* beta = 1.2                                         */
    double minimum_gustiness;            /* 0.01                                               */
    double constant_subgrid_velocity;    /* for NESF_SUBGRID_CONSTANT                          */
    double mesoscale_subgrid_velocity;   /* static mesoscale slot (0 = nothing)                */
    nesf_stability_function stability[3];     /* momentum, temperature, water vapor            */
    nesf_roughness_length roughness[3];       /* momentum, temperature, water vapor            */
    double zero_plane_displacement;      /* d = 0                                              */
    int32_t stop_kind;                   /* nesf_stop_kind                                     */
    int32_t maxiter;                     /* ConvergenceStopCriteria.maxiter or FixedIterations */
    double tolerance;                    /* absolute drift tolerance 1e-8                      */
} nesf_similarity_theory_fluxes;

/* ---------------------------------------------------- CoefficientBasedFluxes
 * coefficient_based_turbulent_fluxes.jl:142-371: bulk transfer coefficients,
 * either constant (Cd, Ch, Cq) or LargeYeagerTransferCoefficients (:82-108): the
 * PolynomialNeutralDragCoefficient (:20-54) with the Large & Yeager (2004)
 * stability corrections (:288-340), whose stability functions are
 * large_yeager_stability_functions (similarity_theory_turbulent_fluxes.jl:766-771).
 * The fixed point is the same iteration (compute_interface_state.jl) with this
 * formulation's stop criteria (ConvergenceStopCriteria(1e-8, 20) by default). */
typedef enum { NESF_FLUXES_SIMILARITY_THEORY = 0, NESF_FLUXES_COEFFICIENT_BASED = 1 } nesf_flux_formulation;
typedef enum { NESF_COEFFICIENTS_CONSTANT = 0, NESF_COEFFICIENTS_LARGE_YEAGER = 1 } nesf_coefficients_kind;

typedef struct {
    int32_t kind;                              /* nesf_coefficients_kind                  */
    int32_t stop_kind;                         /* nesf_stop_kind                          */
    int32_t maxiter;                           /* 20                                      */
    int32_t polynomial_mask;                   /* CONSTANT: bit i set = coefficient i (Cd,
                                                  Ch, Cq) is the PolynomialNeutralDragCoefficient
                                                  of the wind speed (:271), not a number  */
    double tolerance;                          /* 1e-8                                    */
    double momentum, temperature, water_vapor; /* constant Cd, Ch, Cq (1e-3 each)        */
    double von_karman_constant;                /* Large-Yeager: 0.4                       */
    double drag_a, drag_b, drag_c, drag_d;     /* 2.7, 0.142, 1/13.09, 3.14807e-10        */
    double high_wind_speed_threshold;          /* 33                                      */
    double high_wind_drag_coefficient;         /* 2.34e-3                                 */
    double minimum_wind_speed;                 /* 0.5                                     */
    double reference_height;                   /* 10                                      */
    double stable_heat_transfer_coefficient;   /* 18                                      */
    double unstable_heat_transfer_coefficient; /* 32.7                                    */
    double moisture_transfer_coefficient;      /* 34.6                                    */
    nesf_stability_function stability[2];      /* momentum, scalar (linear + Paulson)     */
} nesf_coefficient_fluxes;

/* ------------------------------------------------- surface humidity models
 * interface_states.jl:20-90 (ImpureSaturationSpecificHumidity: ocean, sea ice),
 * 100-230, 587-651 (land: BulkHumidity, FractionalHumidity, SkinHumidity) and
 * dry_layer_humidity.jl:216-366 (land: DryLayerHumidity). */
typedef enum {
    NESF_HUMIDITY_IMPURE_SATURATION = 0,   /* x_H2O e_sat(T_s) (the default)                     */
    NESF_HUMIDITY_BULK = 1,                /* q_sat(T_s) where the land saturation > 0, else 0   */
    NESF_HUMIDITY_FRACTIONAL = 2,          /* beta q_sat(T_s): beta a constant, or
                                              min(S / S_c, 1) (CriticalSaturation)              */
    NESF_HUMIDITY_SKIN = 3,                /* vapor-flux balance with the soil reservoir at the
                                              bulk land temperature (iterated with the fluxes)   */
    NESF_HUMIDITY_DRY_LAYER = 4            /* vapor-flux balance across a dry surface layer whose
                                              depth follows the land saturation, blended with the
                                              saturated skin (iterated with the fluxes)          */
} nesf_humidity_formulation;

/* DryLayerVaporPistonVelocity's tortuosity (dry_layer_humidity.jl:111-127, 252-263). */
typedef enum {
    NESF_TORTUOSITY_CONSTANT = 0,          /* D_eff = D_0                                        */
    NESF_TORTUOSITY_POWER_LAW = 1          /* Millington-Quirk: D_0 theta_g^(10/3) / nu^2        */
} nesf_tortuosity;

/* ------------------------------------------- interface + component properties */
typedef enum { NESF_PHASE_LIQUID = 0, NESF_PHASE_ICE = 1 } nesf_phase;
typedef enum { NESF_RELATIVE_VELOCITY = 0, NESF_WIND_VELOCITY = 1 } nesf_velocity_formulation;
typedef enum {
    NESF_BULK_TEMPERATURE = 0,             /* interface_states.jl:330-333            */
    NESF_SKIN_TEMPERATURE_CONDUCTIVE = 1,  /* ice/snow: interface_states.jl:468-524  */
    NESF_SKIN_TEMPERATURE_DIFFUSIVE = 2    /* ocean DiffusiveFlux: interface_states.jl:434-457 */
} nesf_temperature_formulation;

typedef struct {
    nesf_similarity_theory_fluxes fluxes;
    nesf_thermodynamics_parameters thermo;
    int32_t humidity_phase;               /* nesf_phase                                  */
    int32_t has_water_mole_fraction;      /* 0: nothing (x = 1)                          */
    double water_mole_fraction;           /* x_H2O = 0.98 for the ocean                  */
    int32_t velocity_formulation;         /* nesf_velocity_formulation                   */
    int32_t temperature_formulation;      /* nesf_temperature_formulation                */
    double max_delta_T;                   /* SkinTemperature max_dT = 5                  */
    double ice_conductivity;              /* 2    (ConductiveFlux)                       */
    double snow_conductivity;             /* 0.31 (IceSnowConductiveFlux); 0 = no snow   */
    double diffusive_kappa, diffusive_delta;  /* DiffusiveFlux(kappa, delta)            */
    double gravitational_acceleration;    /* atmosphere_properties g = 9.80665           */
    double surface_layer_height;          /* h    = 10                                   */
    double boundary_layer_height;         /* h_bl = 512                                  */
    double interior_temperature_offset;   /* 273.15: interior temperatures in Celsius    */
    double interface_temperature_offset;  /* 273.15: interface temperature field in C    */
    int32_t has_radiation;                /* radiation state present                     */
    int32_t pad_;
    double stefan_boltzmann_constant;     /* 5.670374419e-8                              */
    double albedo, emissivity;            /* surface radiation properties                */
    double liquidus_freshwater_melting_temperature;  /* LinearLiquidus: 0 (Celsius)     */
    double liquidus_slope;                           /* 0.054                           */
    double interior_reference_density;    /* rho_o (ocean skin temperature)             */
    double interior_heat_capacity;        /* c_o                                         */
    int32_t flux_formulation;             /* nesf_flux_formulation (similarity theory)   */
    int32_t pad2_;
    nesf_coefficient_fluxes coefficients; /* when flux_formulation is coefficient-based */
    int32_t humidity_formulation;         /* nesf_humidity_formulation                   */
    int32_t pad3_;
    double evaporation_efficiency;        /* FRACTIONAL: constant beta (used when
                                             critical_saturation <= 0)                   */
    double critical_saturation;           /* FRACTIONAL: CriticalSaturation S_c (> 0)    */
    double skin_surface_thickness;        /* SKIN: saturation depth d                    */
    double skin_vapor_diffusivity;        /* SKIN: soil vapor diffusivity kappa_q        */
    /* DRY_LAYER (DryLayerHumidity with StorageBasedDryLayerDepth and
       DryLayerVaporPistonVelocity, dry_layer_humidity.jl:81-100, 155-167, 216-235) */
    int32_t tortuosity;                   /* nesf_tortuosity                             */
    int32_t pad4_;
    double maximum_dry_layer_depth;       /* delta_max (m)                               */
    double dry_layer_onset_saturation;    /* S_c: the dry layer appears below it (> 0)   */
    double dry_layer_exponent;            /* eta (2)                                     */
    double minimum_dry_layer_depth;       /* delta_min (m, > 0)                          */
    double molecular_diffusivity;         /* D_0 (m^2/s)                                 */
    double wet_transition_width;          /* logistic blend width (5 delta_min); 0 = sharp */
    double thermal_exchange_depth;        /* l_T (m, > 0)                                */
    double porosity;                      /* nu (> 0 for the power-law tortuosity)       */
} nesf_interface_params;

/* ------------------------------------------------------ solver precision */
typedef enum {
    NESF_PLAIN_F64 = 0,    /* every iteration in FP64: the drop-in                         */
    NESF_F32_POLISH = 1,   /* FP32 iterations, then an FP64 Newton polish of every cell    */
    NESF_F32_ADAPTIVE = 2  /* as NESF_F32_POLISH, but a cell keeps its FP32 result when
                              each state component converged at FP32 resolution, the
                              fixed-point map contracts by at most fp32_rho and the FP32
                              rounding of its cancelling differences, amplified by
                              1 / (1 - rho), stays within path_tolerance; the others are
                              polished in FP64                                            */
} nesf_precision;

typedef struct {
    int32_t precision;        /* nesf_precision                                        */
    int32_t polish_maxiter;   /* FP64 Newton polish steps at most (default 3; 1-3 are
                                 used by contraction rate)                            */
    int32_t block_size;       /* reserved, ignored: the launch shapes and the pass-1
                                 schedule are the context's tuning (nesf_set_tuning,
                                 nesf_autotune)                                         */
    int32_t schedule;         /* reserved, ignored (see block_size)                     */
    int32_t ctas_per_sm;      /* reserved, ignored (see block_size)                     */
    int32_t warm_start;       /* 1: MLP initial guess (needs mlp weights)              */
    const void* mlp;          /* device pointer to packed MLP weights (nesf_mlp_*)      */
    double fallback_ratio;    /* warm start: back to the cold start when the first residual
                                 relative to the state exceeds ratio times the cold start's
                                 relative first residual; 10                            */
    double path_tolerance;    /* replay cells whose reference stopping error may exceed
                                 this relative bound (FP32 polish); default 2e-6         */
    double fp32_rho;          /* NESF_F32_ADAPTIVE: largest contraction rate at which the
                                 FP32 result is kept; default 0.9 (0 or less: default)  */
    double calm_replay_wind;  /* NESF_F32_ADAPTIVE, atmosphere-sea-ice solve: cells whose
                                 10 m wind speed is below it go from the classify pass
                                 straight to the reference's FP64 iteration, on a stream
                                 of their own beside pass 1 when the tuning's two_lanes
                                 is on, else with pass 1's replays (in calm air the fixed
                                 point converges slowly: these are the solve's longest
                                 FP64 chains); default 0: none (measured on the 1/8-degree
                                 step: 0.7 m/s replays more cells in FP64 than pass 1
                                 would, beside pass 1, and the step takes 0.5 ms longer)   */
} nesf_solver_options;

/* -------------------------------------------------------------- statistics */
#define NESF_ITER_HIST_BINS 128
typedef struct {
    int64_t cells;              /* cells visited                                   */
    int64_t solved;             /* cells that ran the fixed point                  */
    int64_t iterations;         /* sum of iterations over solved cells             */
    int64_t max_iterations;
    int64_t nonconverged;       /* cells that stopped at maxiter                   */
    int64_t polished;           /* cells that needed an FP64 polish                */
    int64_t polish_iterations;  /* FP64 polish iterations                          */
    int64_t cold_fallbacks;     /* warm starts rejected by the residual test       */
    int64_t fp64_redo;          /* cells replayed in FP64 (sum of replay_reasons)  */
    int64_t replay_reasons[5];  /* calm u*, no FP32 convergence, slow contraction,
                                   stopping-error bound, singular Newton matrix   */
    int64_t histogram[NESF_ITER_HIST_BINS]; /* iterations (FP32+FP64) per solved cell */
} nesf_stats;

/* ------------------------------------------- atmosphere-ocean field bundle
 * Arguments of _compute_atmosphere_ocean_interface_state!
 * (atmosphere_ocean_fluxes.jl:80-197) */
typedef struct {
    nesf_grid grid;
    int32_t dtype;                 /* nesf_dtype of every float array below               */
    int32_t pad_;
    const void* u_atm;  const void* v_atm;  const void* T_atm;  const void* p_atm;  const void* q_atm;
    const void* u_oc;              /* ocean u at k = Nz (x-face)                          */
    const void* v_oc;              /* ocean v at k = Nz (y-face)                          */
    const void* T_oc;              /* ocean T at k = Nz (interior temperature units)     */
    const void* S_oc;              /* ocean S at k = Nz                                   */
    const uint8_t* inactive;       /* 1 = land/immersed (halo included); NULL = none      */
    const void* sw_down;           /* downwelling shortwave (skin formulations only)      */
    const void* lw_down;           /* downwelling longwave                                */
    const void* kappa;             /* interior diffusivity (InteriorDiffusivity) or NULL  */
    /* outputs: AtmosphereSurfaceFluxes (component_interfaces.jl:69-78) + T_s */
    void* latent_heat; void* sensible_heat; void* water_vapor;
    void* x_momentum;  void* y_momentum;
    void* friction_velocity; void* temperature_scale; void* water_vapor_scale;
    void* interface_temperature;
    int32_t* iterations;           /* optional: iterations per cell (same layout)         */
} nesf_ao_fields;

/* ------------------------------------------------ atmosphere-land bundle
 * _compute_atmosphere_land_interface_state! (atmosphere_land_fluxes.jl:146-251):
 * interior cells, surface velocities zero, T_s starts at (BulkTemperature: is) the
 * bulk land temperature, in kelvin (the interface params' temperature offsets
 * are not applied to land). */
typedef struct {
    nesf_grid grid;
    int32_t dtype;
    int32_t pad_;
    const void* u_atm; const void* v_atm; const void* T_atm; const void* p_atm; const void* q_atm;
    const void* land_temperature;      /* bulk land temperature T (K)                          */
    const void* saturation;            /* land surface saturation S (BULK, DRY_LAYER,
                                          FRACTIONAL with S_c)                                 */
    /* outputs: AtmosphereSurfaceFluxes + T_s */
    void* latent_heat; void* sensible_heat; void* water_vapor;
    void* x_momentum;  void* y_momentum;
    void* friction_velocity; void* temperature_scale; void* water_vapor_scale;
    void* interface_temperature;
    int32_t* iterations;
} nesf_al_fields;

/* --------------------------------------------- atmosphere-sea-ice bundle
 * _compute_atmosphere_sea_ice_interface_state! (atmosphere_sea_ice_fluxes.jl:65-185) */
typedef struct {
    nesf_grid grid;
    int32_t dtype;
    int32_t pad_;
    const void* u_atm; const void* v_atm; const void* T_atm; const void* p_atm; const void* q_atm;
    const void* T_oc; const void* S_oc;          /* ocean surface under the ice         */
    const void* ice_thickness;                   /* h_i                                 */
    const void* snow_thickness;                  /* h_s (NULL = no snow)                */
    const void* consolidation_thickness;         /* h_c                                 */
    const void* ice_concentration;               /* aleph                               */
    const uint8_t* inactive;
    const void* sw_down; const void* lw_down;
    /* in/out: interface (top surface) temperature; read as the initial T_s */
    void* interface_temperature;
    /* outputs: AtmosphereSeaIceFluxes (component_interfaces.jl:111-117) */
    void* latent_heat; void* sensible_heat; void* water_vapor; void* x_momentum; void* y_momentum;
    int32_t* iterations;
} nesf_ai_fields;

/* ----------------------------------------------------- sea-ice-ocean bundle
 * sea_ice_ocean_fluxes.jl:106-226 + sea_ice_ocean_heat_flux_formulations.jl:118-313 */
typedef struct {
    int32_t formulation;            /* 0: ThreeEquationHeatFlux; 1: IceBathHeatFlux        */
    int32_t conductive;             /* ThreeEquation with ConductiveFlux internal flux      */
    double heat_transfer_coefficient;   /* alpha_h 0.0095 (IceBath 0.006)                 */
    double salt_transfer_coefficient;   /* alpha_s = alpha_h / 35                         */
    double friction_velocity;           /* constant u* 0.002                              */
    double ice_conductivity;            /* k for ConductiveFlux                           */
    double reference_latent_heat;       /* phase_transitions.reference_latent_heat        */
    double liquidus_freshwater_melting_temperature, liquidus_slope;
    double ocean_reference_density, ocean_heat_capacity;
    double dt;                          /* sea-ice time step                               */
    int32_t nz;                         /* ocean levels for the frazil column             */
    int32_t pad_;
    int64_t stride_k;                   /* elements between levels of the 3-D T/S arrays  */
} nesf_io_params;

typedef struct {
    nesf_grid grid;
    int32_t dtype;
    int32_t pad_;
    void* T_oc;                      /* 3-D ocean temperature, pointer of level k = 1 (mutated by frazil) */
    const void* S_oc;                /* 3-D ocean salinity, pointer of level k = 1                         */
    const double* dz;                /* host or device? device array of nz layer thicknesses              */
    const void* ice_salinity; const void* ice_thickness; const void* consolidation_thickness;
    const void* ice_concentration;
    const void* internal_temperature;   /* ice top temperature (ConductiveFlux formulation)  */
    const void* ice_mass_flux; const void* snow_mass_flux;
    /* outputs: SeaIceOceanFluxes (component_interfaces.jl:143-150) + interface T, S */
    void* interface_heat; void* frazil_heat; void* salt; void* freshwater;
    void* interface_T; void* interface_S;
} nesf_io_fields;

/* ----------------------------------------------- prescribed atmosphere
 * PrescribedAtmosphere on a regular longitude-latitude grid, two time levels */
typedef struct {
    int32_t nx, ny;                   /* atmosphere interior size                        */
    int32_t hx, hy;
    int64_t stride_j;
    int64_t stride_t;                 /* elements between the two time snapshots          */
    double lon0, dlon;                /* longitude of the first cell centre, spacing      */
    double lat0, dlat;                /* latitude of the first cell centre, spacing       */
} nesf_atmos_grid;

typedef struct {
    double lon0, dlon, lat0, dlat;    /* exchange grid: first cell centre and spacing     */
} nesf_exchange_coords;

typedef struct {
    nesf_grid grid;                   /* exchange grid layout                              */
    nesf_exchange_coords coords;
    nesf_atmos_grid atmos;
    int32_t dtype;                    /* dtype of atmosphere AND exchange arrays           */
    int32_t pad_;
    double time_weight;               /* n~ in [0, 1] between snapshot 1 and 2            */
    const void* u; const void* v; const void* T; const void* q; const void* p;
    const void* rain; const void* snow;           /* may be NULL (zero)                    */
    const void* sw_down; const void* lw_down;     /* radiation; may be NULL                */
    /* exchange-grid outputs (NULL skips the variable) */
    void* u_out; void* v_out; void* T_out; void* q_out; void* p_out;
    void* rain_out; void* snow_out; void* sw_out; void* lw_out;
    /* optional fractional-index cache, FP64, exchange layout; NULL = recompute inline */
    const double* frac_i; const double* frac_j;
} nesf_interp_fields;

/* ----------------------------------------------- time interpolation of forcing
 * The time indexing of Oceananigans' FieldTimeSeries, which PrescribedAtmosphere holds its
 * forcing in (cpu_interpolating_time_indices, as interpolate_atmospheric_state.jl:57-60
 * calls it; the JRA55 atmosphere cycles its repeat year,
 * JRA55_prescribed_atmosphere.jl:37). Host-only: no device work. */
typedef enum {
    NESF_TIME_CYCLICAL = 0,   /* t wrapped into [t_0, t_0 + period); between t_last and
                                 t_0 + period the last snapshot blends into the first        */
    NESF_TIME_LINEAR = 1,     /* the bracketing interval, extrapolated beyond the ends        */
    NESF_TIME_CLAMP = 2       /* the first / last snapshot outside the range                  */
} nesf_time_indexing;

/* The snapshots n1, n2 (0-based) that bracket time t and the weight of n2 (the
   interpolation's time_weight). times: nt strictly increasing values; period: the cycle
   length for NESF_TIME_CYCLICAL (<= 0: t_last - t_0 plus the last interval). */
int nesf_time_indices(const double* times, int32_t nt, int32_t indexing, double period, double t, int32_t* n1,
                      int32_t* n2, double* weight);

/* ------------------------------------------------------- net-flux assembly */
typedef struct {
    double ocean_reference_density;   /* rho_o */
    double ocean_heat_capacity;       /* c_o   */
    double interface_temperature_offset;   /* 273.15 when T_s is stored in Celsius */
    double stefan_boltzmann_constant;
    double ocean_albedo, ocean_emissivity;
    double ice_albedo, ice_emissivity;
} nesf_assembly_params;

typedef struct {
    nesf_grid grid;
    int32_t dtype;
    int32_t pad_;
    const uint8_t* inactive;
    const void* ice_concentration;                   /* NULL = no sea ice               */
    const void* ocean_surface_temperature;           /* T_oc at k = Nz (Celsius)        */
    const void* rain; const void* snow; const void* intercepted_snow; const void* land_freshwater;
    /* atmosphere-ocean fluxes */
    const void* ao_sensible; const void* ao_latent; const void* ao_water_vapor;
    const void* ao_x_momentum; const void* ao_y_momentum;
    const void* ao_interface_temperature;
    /* sea-ice-ocean fluxes (NULL = none) */
    const void* io_interface_heat; const void* io_frazil_heat; const void* io_salt;
    const void* io_freshwater; const void* io_x_momentum; const void* io_y_momentum;
    /* atmosphere-sea-ice fluxes (NULL = none) */
    const void* ai_sensible; const void* ai_latent; const void* ai_x_momentum; const void* ai_y_momentum;
    const void* ai_interface_temperature;
    /* radiation (NULL = no radiation) */
    const void* sw_down; const void* lw_down;
    /* outputs: net ocean fluxes (Oceans.jl:174-191) */
    void* ocean_u; void* ocean_v; void* ocean_T; void* ocean_S; void* ocean_eta; void* ocean_heat_content;
    /* outputs: net sea-ice fluxes (sea_ice_simulation.jl:223-237) */
    void* ice_top_heat; void* ice_top_snowfall; void* ice_top_u; void* ice_top_v; void* ice_bottom_heat;
    /* optional radiation diagnostics (InterfaceRadiationFlux) */
    void* ocean_upwelling_longwave; void* ocean_downwelling_longwave; void* ocean_downwelling_shortwave;
    void* ice_upwelling_longwave; void* ice_downwelling_longwave; void* ice_downwelling_shortwave;
} nesf_assembly_fields;

/* ------------------------------------------ land net-flux assembly and radiation
 * update_net_fluxes!(model, land::SlabLand) (Lands/slab_land.jl:285-329) and
 * apply_air_land_radiative_fluxes! (Radiations/apply_air_land_radiative_fluxes.jl:22-95)
 * over the land exchange grid's interior. */
typedef struct {
    double stefan_boltzmann_constant;     /* 5.670374419e-8                               */
    double land_albedo, land_emissivity;  /* the radiation's land SurfaceRadiationProperties
                                             (the reference has no default: land_surface =
                                             nothing means no land radiation)             */
} nesf_land_radiation_params;

typedef struct {
    nesf_grid grid;                       /* the land grid                                */
    int32_t dtype;
    int32_t pad_;
    const uint8_t* inactive;              /* radiation only; NULL = every cell active     */
    const void* rain;                     /* the atmosphere exchanger's rainfall; NULL = 0 */
    /* atmosphere-land fluxes (nesf_compute_atmosphere_land_fluxes outputs) */
    const void* al_sensible; const void* al_latent; const void* al_water_vapor;
    const void* al_interface_temperature; /* T_s (kelvin)                                  */
    const void* sw_down; const void* lw_down;   /* radiation                              */
    /* outputs, the SlabLand flux accumulators (NULL skips one) */
    void* surface_energy_flux;            /* Q_T + Q_v, positive upward; the radiation adds
                                             sigma eps T_s^4 - eps LW - (1 - alpha) SW    */
    void* precipitation;                  /* rain + max(0, -J_v)                          */
    void* evaporation;                    /* max(0, J_v)                                  */
    void* vapor_flux;                     /* J_v                                          */
    void* liquid_precipitation_flux;      /* rain                                         */
    /* radiation diagnostics (InterfaceRadiationFlux of the land; NULL skips one) */
    void* upwelling_longwave; void* downwelling_longwave; void* downwelling_shortwave;
} nesf_land_flux_fields;

/* ------------------------------------------------ area integrals (FP64)
 * The global flux integrals behind the reference's conservation checks,
 * int dA(a) = sum(a) * A_z and int dA(a, b) = sum(a .* b) * A_z
 * (test/test_conservation.jl:100-101), over the interior cells, as compensated
 * FP64 sums: each integral is returned as a pair (sum, residual) whose sum is the
 * exact sum of the cell terms to ~1e-30 relative. Cell term: a (times b when
 * `factor` is given) times the cell area (`area`, 2-D FP64 in the parent layout, or
 * `row_area`, ny FP64 entries for j = 1..ny), products rounded in FP64; with
 * neither, the sum is multiplied by `uniform_area` at the end, as the reference
 * does. Cells with inactive != 0 are skipped when `inactive` is given. The
 * reduction order is fixed: the result is the same on every run. */
#define NESF_MAX_INTEGRALS 16
typedef struct {
    nesf_grid grid;
    int32_t dtype;                                /* nesf_dtype of field[] and factor[] */
    int32_t n;                                    /* integrals, 1..NESF_MAX_INTEGRALS  */
    const void* field[NESF_MAX_INTEGRALS];
    const void* factor[NESF_MAX_INTEGRALS];       /* NULL: no second factor            */
    const uint8_t* inactive;
    const double* area;
    const double* row_area;
    double uniform_area;
} nesf_integral_fields;

/* ------------------------------------------------------------------ API */
/* Library-owned scratch per device, grown on demand to the largest grid solved: per
   halo-ring cell the work list and replay queue (uint32 each), under NESF_F32_ADAPTIVE a
   64-byte record of pass 1's cancelling differences, with the warm start 48 bytes of
   features and guesses (the 1/8-degree coupled step, 3.7 M ring cells: about 0.5 GB on
   the caller's context and up to as much on the sea-ice lane's). */
typedef struct nesf_context nesf_context;

int32_t     nesf_abi_version(void);
const char* nesf_version(void);
/* Per-device set-up ahead of the first call (the default context that calls with a
   null context use); optional, the first call does it otherwise. */
int nesf_init(int32_t device);
const char* nesf_last_error(void);
/* sizes of the public structs, for binding checks: fills n entries */
int32_t     nesf_struct_sizes(int64_t* sizes, int32_t n);

/* Fill parameter structs with the reference defaults (host memory). */
void nesf_default_thermodynamics(nesf_thermodynamics_parameters* p);
void nesf_default_ao_params(nesf_interface_params* p);      /* ComponentInterfaces AO defaults */
void nesf_default_ai_params(nesf_interface_params* p);      /* AO defaults + ice/skin changes  */
/* CoefficientBasedFluxes defaults (coefficient_based_turbulent_fluxes.jl:30-37,92-99,215-229) for
 * transfer coefficients of `kind`; put in params->coefficients with flux_formulation
 * NESF_FLUXES_COEFFICIENT_BASED. */
void nesf_default_coefficient_fluxes(nesf_coefficient_fluxes* c, int32_t kind);
/* Atmosphere-land defaults (component_interfaces.jl:404-406, 501-521):
 * SimilarityTheoryFluxes with large_yeager_stability_functions and constant
 * roughness lengths 0.1 m (momentum) / 0.01 m (scalars), BulkTemperature,
 * RelativeVelocity, BulkHumidity(Liquid); temperatures in kelvin. */
void nesf_default_al_params(nesf_interface_params* p);
void nesf_default_io_params(nesf_io_params* p);
void nesf_default_assembly_params(nesf_assembly_params* p);
void nesf_default_solver_options(nesf_solver_options* o);

int nesf_context_create(int32_t device, nesf_context** ctx);
int nesf_context_destroy(nesf_context* ctx);

/* compute_atmosphere_ocean_fluxes! (atmosphere_ocean_fluxes.jl:17-60):
 * launches over the halo ring (0:nx+1, 0:ny+1) like interface_kernel_parameters
 * (InterfaceComputations.jl:100-116). */
int nesf_compute_atmosphere_ocean_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                         const nesf_ao_fields* fields, const nesf_solver_options* opts,
                                         nesf_stats* stats, void* stream);

/* Ensemble variant: `members` independent copies of the AO problem laid out
 * back to back (member stride `member_stride` elements in every array), each
 * with its own parameters (`params[members]`, host memory). */
int nesf_compute_atmosphere_ocean_fluxes_ensemble(nesf_context* ctx, const nesf_interface_params* params,
                                                  int32_t members, int64_t member_stride,
                                                  const nesf_ao_fields* fields, const nesf_solver_options* opts,
                                                  nesf_stats* stats, void* stream);

/* The atmosphere-ocean solve without any device allocation, for callers that
 * cannot allocate at call time (a host model whose pooling allocator holds the
 * whole device, or a caller that must not enter the driver's allocator). No
 * counterpart in the reference. Its scratch is a fixed 24 MiB array in the
 * library, shared by every call: grids of more than 2,097,152 cells (halo ring
 * (nx+2) x (ny+2)) are rejected with NESF_ERR_CAPACITY; calls that overlap on the
 * GPU race on the scratch. The device must have been prepared with
 * nesf_noalloc_prepare (else NESF_ERR_ARG). No warm start (NESF_ERR_ARG if
 * requested), no statistics; the context's tuning is not used (default launch
 * shapes). Under NESF_F32_ADAPTIVE its pass 1 forms the cancelling differences
 * (theta_a - T_s, q_a - q_s ...) in FP64 in the kernel, where the regular entry
 * point reads them from per-cell double-float records of its classify pass (a
 * scratch of 64 bytes per cell): the two FP32 trajectories then differ and the
 * results agree within the solver's tolerance, not bit for bit. */
int nesf_compute_atmosphere_ocean_fluxes_noalloc(const nesf_interface_params* params, const nesf_ao_fields* fields,
                                                 const nesf_solver_options* opts, void* stream);
/* Set-up of the allocation-free solve on `device`, once, at the caller's set-up:
 * it loads the library's module holding the 24 MiB scratch array (under lazy
 * module loading a device reserves that memory only then) and every kernel the
 * solve can launch, and resolves the array's device address. Call it before the
 * host's memory pool reserves the device and before any stream capture; the
 * device holds the array until the process exits. No counterpart in the reference. */
int nesf_noalloc_prepare(int32_t device);

/* compute_atmosphere_sea_ice_fluxes! (atmosphere_sea_ice_fluxes.jl:18-62) */
int nesf_compute_atmosphere_sea_ice_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                           const nesf_ai_fields* fields, const nesf_solver_options* opts,
                                           nesf_stats* stats, void* stream);
/* compute_atmosphere_land_fluxes! (atmosphere_land_fluxes.jl:48-105). The FP32 modes
 * apply to the BULK, FRACTIONAL and IMPURE_SATURATION humidity models (FP32 sweep +
 * FP64 polish, FP64 replays in place); SKIN humidity, whose surface humidity is
 * part of the iterated state, always runs the FP64 iteration. Default parameters:
 * nesf_default_al_params. */
int nesf_compute_atmosphere_land_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                        const nesf_al_fields* fields, const nesf_solver_options* opts,
                                        nesf_stats* stats, void* stream);

/* compute_sea_ice_ocean_fluxes! (sea_ice_ocean_fluxes.jl:33-77): interior (:xy) launch */
int nesf_compute_sea_ice_ocean_fluxes(nesf_context* ctx, const nesf_io_params* params,
                                      const nesf_io_fields* fields, void* stream);

/* initialize!(exchanger) -> _compute_fractional_indices! (prescribed_atmosphere_regridder.jl:41-71) */
int nesf_compute_fractional_indices(const nesf_grid* grid, const nesf_exchange_coords* coords,
                                    const nesf_atmos_grid* atmos, double* frac_i, double* frac_j,
                                    void* stream);

/* interpolate_state!(exchanger, grid, ::PrescribedAtmosphere, model)
 * (interpolate_atmospheric_state.jl:9-137) and the radiation twin
 * (interpolate_radiation_state.jl:4-69): halo-ring launch. */
int nesf_interpolate_atmosphere_state(const nesf_interp_fields* fields, void* stream);

/* update_net_fluxes!(model, ocean) (assemble_net_ocean_fluxes.jl:30-153) */
int nesf_assemble_net_ocean_fluxes(const nesf_assembly_params* params, const nesf_assembly_fields* fields,
                                   void* stream);
/* update_net_fluxes!(model, sea_ice) (assemble_net_sea_ice_fluxes.jl:11-81) */
int nesf_assemble_net_sea_ice_fluxes(const nesf_assembly_params* params, const nesf_assembly_fields* fields,
                                     void* stream);
/* apply_air_sea_radiative_fluxes! (apply_air_sea_radiative_fluxes.jl:18-111) */
int nesf_apply_air_sea_radiative_fluxes(const nesf_assembly_params* params, const nesf_assembly_fields* fields,
                                        void* stream);
/* apply_air_sea_ice_radiative_fluxes! (apply_air_sea_ice_radiative_fluxes.jl:15-90) */
int nesf_apply_air_sea_ice_radiative_fluxes(const nesf_assembly_params* params, const nesf_assembly_fields* fields,
                                            void* stream);
/* update_net_fluxes!(model, land::SlabLand) (Lands/slab_land.jl:285-329): the SlabLand flux
   accumulators from the atmosphere-land fluxes and the rainfall */
int nesf_assemble_net_land_fluxes(const nesf_land_flux_fields* fields, void* stream);
/* apply_air_land_radiative_fluxes! (Radiations/apply_air_land_radiative_fluxes.jl:22-95): the
   radiative part added in place to surface_energy_flux, and the diagnostics */
int nesf_apply_air_land_radiative_fluxes(const nesf_land_radiation_params* params, const nesf_land_flux_fields* fields,
                                         void* stream);

/* int dA of up to 16 fields; result: device memory, 2 n doubles (sum, residual) per
 * integral, written on `stream`. */
int nesf_area_integrals(nesf_context* ctx, const nesf_integral_fields* fields, double* result, void* stream);

/* ------------------------------------------------------ double-float check
 * The adaptive solver's FP64 replays of the cells its FP32 sweep does not keep run in
 * double-float arithmetic (a value as the unevaluated sum of two FP32 numbers, 48
 * significant bits) on the FP32 pipes: this GPU issues one FP64 warp instruction per
 * ~64 cycles per SM sub-partition. This entry point checks that arithmetic: out[i] =
 * op(x[i], y[i]) (y only for the binary operations) with the arguments rounded to
 * double-float and the result widened to FP64; x, y, out device arrays of n doubles,
 * launched on `stream` (not synchronised). No counterpart in the reference. */
enum {
    NESF_DF_ADD = 0, NESF_DF_SUB = 1, NESF_DF_MUL = 2, NESF_DF_DIV = 3, NESF_DF_SQRT = 4, NESF_DF_CBRT = 5,
    NESF_DF_EXP = 6, NESF_DF_LOG = 7, NESF_DF_POW = 8, NESF_DF_ATAN = 9
};
int nesf_double_float_check(const double* x, const double* y, double* out, int64_t n, int32_t op, void* stream);

/* ------------------------------------------------------ tensor-core check
 * Self-check of the tcgen05 GEMM building blocks of the warm-start network in the
 * three operand arrangements it uses (BF16 in, FP32 out; a, b, d device memory,
 * row-major): which = 0: d[128x64] = a[128x64] b[64x64]^T; which = 1:
 * d[128x64] = a[128x64] b[64x64]; which = 2: d[128x16] = a[128x128]^T b[128x16].
 * which = 3 checks the failure path instead: no MMA is issued, so the kernel's
 * bounded wait on its mbarrier gives up after 64 polls, records the error, frees
 * its TMEM and returns; the call returns NESF_ERR_TIMEOUT and the context stays
 * usable (d is not written).
 * Synchronises the stream; NESF_ERR_TIMEOUT if the MMA did not complete. */
int nesf_mlp_selftest(const void* a, const void* b, float* d, int32_t which, void* stream);

/* ------------------------------------------------- learned warm start
 * A 6 -> 64 -> 64 -> 3 GELU network that predicts the transfer coefficients
 * c_u = u* / dU, c_theta = theta* / dtheta_0, c_q = q* / dq_0 of a cell's fixed
 * point from six features of its state before the iteration (bulk Richardson
 * number, dU, dtheta_0, dq_0, ln h, ln of a neutral roughness). Its parameters live
 * in one device blob of nesf_mlp_bytes() bytes (FP32 masters, BF16 copies, the
 * gradient and the Adam moments); inference and training run on the tensor cores
 * (tcgen05, BF16 operands, FP32 accumulation). Features are 8 floats per sample
 * (6 used; the feature array 16-byte aligned), targets 4 (c_u, c_theta, c_q, and a
 * bit mask of the valid ones as a float), outputs 4 (c_u, c_theta, c_q, 1); inference
 * evaluates GELU with the hardware's tanh approximation (its activations are BF16
 * anyway), training with tanhf. The solvers take a trained blob through
 * nesf_solver_options.mlp with warm_start = 1 (FP32 modes, single member, bulk
 * interface temperature: a skin temperature keeps the reference's start). No
 * counterpart in the reference. */
typedef struct {
    int32_t epochs;
    int32_t batch;              /* samples per Adam step (a multiple of 128) */
    float learning_rate, beta1, beta2, eps;
} nesf_mlp_train_options;

int64_t nesf_mlp_bytes(void);
int nesf_mlp_init(void* mlp, uint64_t seed, void* stream);
/* Feature and target means and deviations from a sample set (stored in the blob). */
int nesf_mlp_fit_normalization(void* mlp, const float* features, const float* targets, int64_t n, void* stream);
/* Adds the gradient of the mean squared error of the n samples (normalised
 * targets) to the blob's gradient and the error sum to its loss slots. */
int nesf_mlp_gradient(void* mlp, const float* features, const float* targets, int64_t n, void* stream);
/* Mini-batch Adam over the samples; `loss` (host, epochs entries, may be NULL)
 * receives the mean loss of each epoch (synchronises the stream once per epoch). */
int nesf_mlp_train(void* mlp, const float* features, const float* targets, int64_t n,
                   const nesf_mlp_train_options* opts, float* loss, void* stream);
int nesf_mlp_infer(void* mlp, const float* features, int64_t n, float* out, void* stream);
/* Training samples from an atmosphere-ocean state: the features of every
 * halo-ring cell (ring order, 8 floats: the 6 network inputs, then dU again and 0)
 * and, when `targets` is given, the targets of the solved state in the fields'
 * friction_velocity, temperature_scale and water_vapor_scale outputs. Land cells,
 * and coefficients whose scale is near zero (|dtheta_0| < 0.05 K, |dq_0| < 1e-5),
 * are masked out. */
int nesf_mlp_ao_samples(const nesf_interface_params* params, const nesf_ao_fields* fields, float* features,
                        float* targets, void* stream);

/* ------------------------------------------------------- the coupling step
 * The interface-flux part of update_state!(::EarthSystemModel)
 * (EarthSystemModels/time_step_earth_system_model.jl:38-83) in one call, in the
 * reference's order: interpolate_state! (when `interp` is given),
 * compute_atmosphere_ocean_fluxes!, compute_atmosphere_sea_ice_fluxes! and
 * compute_sea_ice_ocean_fluxes! (when their parameters are given),
 * update_net_fluxes! for the ocean and the sea ice (when `assembly_params` is
 * given; the sea-ice half only with sea ice), then the radiative add-ons (when
 * `radiation` is 1). The pointers of one phase's fields must agree with the
 * arrays the next phase reads (a model's fields); nothing is checked across
 * phases. No statistics. */
typedef struct {
    const nesf_interface_params* ao_params;         /* required                          */
    const nesf_ao_fields* ao;                       /* required                          */
    const nesf_interface_params* ai_params;         /* NULL: no sea ice                  */
    const nesf_ai_fields* ai;
    const nesf_io_params* io_params;                /* NULL: no sea-ice-ocean fluxes     */
    const nesf_io_fields* io;
    const nesf_interp_fields* interp;               /* NULL: exchange-grid state given   */
    const nesf_assembly_params* assembly_params;    /* NULL: no net-flux assembly        */
    const nesf_assembly_fields* assembly;
    int32_t radiation;                              /* 1: radiative add-ons after assembly
                                                       (inside the assembly kernels: bit for
                                                       bit the separate apply_* calls)     */
    int32_t pad_;
} nesf_coupling_step_args;

int nesf_coupling_step(nesf_context* ctx, const nesf_coupling_step_args* args, const nesf_solver_options* opts,
                       void* stream);

/* A CUDA graph of one coupling step, captured once and replayed each step: the
 * launch sequence (16 kernels and 4 counter resets for a coupled step) becomes one
 * graph launch. Everything the step reads is baked in at capture -- the field
 * pointers, parameters and options -- so the caller keeps its buffers between
 * launches (a model's fields are fixed; new atmosphere snapshots are copied into
 * the captured snapshot arrays). The interpolation's time weight changes every
 * step and is set with nesf_graph_set_time_weight. The graph uses the context's
 * scratch: do not run other solves on the same context concurrently with it.
 * Capture sizes the scratch first (it may synchronise the device then); launches
 * never allocate or synchronise. */
typedef struct nesf_graph nesf_graph;

int nesf_graph_capture(nesf_context* ctx, const nesf_coupling_step_args* args, const nesf_solver_options* opts,
                       nesf_graph** out);
int nesf_graph_set_time_weight(nesf_graph* graph, double time_weight);
int nesf_graph_launch(nesf_graph* graph, void* stream);
/* The snapshot pair the captured interpolation reads, for a forcing window whose pair moves
   between device slots: src[9] (u v T q p rain snow sw lw; NULL keeps the captured array,
   and only variables interpolated at capture can be set) is each variable's first snapshot,
   stride_t the elements from it to the second (negative allowed), time_weight the pair's
   weight (nesf_time_indices). The arrays keep the captured atmosphere grid and dtype. */
int nesf_graph_set_forcing(nesf_graph* graph, const void* const* src, int64_t stride_t, double time_weight);
int nesf_graph_destroy(nesf_graph* graph);

/* ------------------------------------------------------------ the autotuner
 * Launch shapes and schedule of a context's solves and coupling steps. None of
 * them changes a result: every cell's arithmetic is the same under each, so the
 * outputs are bit-identical (the tests check it); only the time differs. 0 in a
 * field means its default. Replaces nothing in the reference (Julia launches its
 * kernels with KernelAbstractions' default workgroup); it is the `nesf_autotune`
 * entry of the GB300 design. */
typedef struct {
    int32_t solve_block;      /* threads per block of the solves' pass 1: 32, 64, 96 or 128 (128)       */
    int32_t deferred_per_sm;  /* blocks per SM of the packed polish and replay passes, 1..16 (4)      */
    int32_t infer_per_sm;     /* blocks per SM of the warm-start inference pass, 1..8 (4)             */
    int32_t two_lanes;        /* coupling step: sea-ice solve on a second stream beside the ocean's (1) */
    int32_t io_overlap;       /* coupling step: sea-ice-ocean fluxes beside the sea-ice pass 1 (1)      */
    int32_t pass1_fetch;      /* pass 1 of the FP32 solvers: 1 one thread per work-list entry; 2 in the
                                 sea-ice solve, 3 in the sea-ice and ocean solves, the resident blocks
                                 only, each warp taking 32 entries at a time; 4 as 3 with lane refill
                                 in the adaptive solver's pass 1: a warp takes new entries for its
                                 idle lanes as soon as refill_lanes of them are idle (2)              */
    int32_t refill_lanes;     /* pass1_fetch 4: idle lanes that make a warp take new entries, 1..32
                                 (32: warp fetching) (8)                                                */
    int32_t early_ocean_classify; /* coupling step with two lanes: the ocean's classify pass and
                                 warm-start inference 0 after the sea-ice pass 1, 1 beside it, 2
                                 before it (the sea-ice pass 1 waits for them), 3 after it with the
                                 sea-ice polish pass waiting for them; the ocean's pass 1 follows
                                 the sea-ice pass 1 in each (0)                                   */
    int32_t ice_deferred_per_sm; /* blocks per SM of the sea-ice solve's packed polish and replay
                                 passes, 1..16; 0: deferred_per_sm. Fewer leave registers to the
                                 ocean solve's kernels that run beside them (0)              */
    int32_t cells_per_thread; /* pass 1 of the adaptive solver, 1..8: work-list entries a thread
                                 takes one after another -- with one thread per entry the grid
                                 shrinks by this factor; with fetching each lane reserves this
                                 many entries per fetch (fewer atomic adds, a longer tail) (1)  */
    double step_ms;           /* nesf_autotune: the chosen configuration's mean step time            */
} nesf_tuning;

/* The context's tuning (a NULL context: the default context's). Fields out of
 * range are an argument error; 0 selects the default. A graph keeps the tuning
 * it was captured with. */
int nesf_set_tuning(nesf_context* ctx, const nesf_tuning* tuning);
int nesf_get_tuning(nesf_context* ctx, nesf_tuning* tuning);
/* Coordinate search over the tuning on the caller's workload: for each field in
 * turn, each candidate value is timed (the step captured as a graph under it, CUDA
 * events on `stream`, one untimed replay, then `reps` replays) with the others at
 * their best so far; the fastest setting is
 * kept. The chosen tuning is set on the context and written to `out` with its
 * step time. The steps run for real: the outputs and the in/out state (sea-ice
 * surface temperature, frazil-adjusted ocean temperature) are left as that many
 * coupling steps leave them. Synchronises `stream`. */
int nesf_autotune(nesf_context* ctx, const nesf_coupling_step_args* args, const nesf_solver_options* opts,
                  int32_t reps, nesf_tuning* out, void* stream);

/* The autotuner's results on disk, so that a model is tuned once per device and
 * workload rather than once per run. A key names what a tuning was measured on; a
 * cache file (any path the caller picks) holds one tuning per key. Format, every
 * integer little-endian whatever the host:
 *   "NESFTUNE" (8 bytes), uint32 format version (NESF_TUNING_VERSION), uint32 key
 *   bytes (108), uint32 tuning fields (10), uint32 record count, then per record the
 *   key (device name, 64 bytes NUL-padded, then its eleven int32 fields) and the
 *   tuning (its ten int32 fields in declaration order, then step_ms as the
 *   IEEE-754 bits of a double).
 * A file of another format version or tuning-field count holds nothing for this
 * library: find reports no entry and store starts the file afresh. A file that does
 * not start with the magic, or is cut short, is an argument error (store does not
 * overwrite it). Store writes `path`.tmp and renames it over `path`; concurrent
 * writers of one path may lose each other's entries. No reference counterpart (the
 * reference has no autotuner). */
#define NESF_TUNING_VERSION 2
typedef struct {
    char device[64];              /* cudaDeviceProp::name, NUL-padded                         */
    int32_t sm_count;             /* multiprocessors                                          */
    int32_t compute_capability;   /* major * 10 + minor                                       */
    int32_t nx, ny;               /* interior grid of the atmosphere-ocean fields             */
    int32_t hx, hy;               /* their halo widths                                        */
    int32_t dtype;                /* nesf_dtype of the fields                                 */
    int32_t precision;            /* nesf_solver_options.precision                            */
    int32_t warm_start;           /* 1: the step runs with a warm-start network               */
    int32_t parts;                /* bit 0 sea ice, 1 sea-ice-ocean fluxes, 2 interpolation,
                                     3 net-flux assembly, 4 radiative add-ons                 */
    int32_t flux_formulation;     /* the atmosphere-ocean params' flux_formulation            */
} nesf_tuning_key;

/* The key of a coupling step on the context's device. */
int nesf_tuning_key_of(nesf_context* ctx, const nesf_coupling_step_args* args, const nesf_solver_options* opts,
                       nesf_tuning_key* key);
/* The cached tuning of `key`: *found = 1 and the tuning in `out`, or *found = 0 (no
 * file, a stale file, or no record of the key). Host only. */
int nesf_tuning_cache_find(const char* path, const nesf_tuning_key* key, nesf_tuning* out, int32_t* found);
/* Record `tuning` for `key` (replacing an earlier record of the key). Host only. */
int nesf_tuning_cache_store(const char* path, const nesf_tuning_key* key, const nesf_tuning* tuning);
/* nesf_autotune through the cache: the cached tuning of this step's key is set on the
 * context without running a step (*from_cache = 1); otherwise the search runs and its
 * result is stored (*from_cache = 0). */
int nesf_autotune_cached(nesf_context* ctx, const nesf_coupling_step_args* args, const nesf_solver_options* opts,
                         int32_t reps, const char* path, nesf_tuning* out, int32_t* from_cache, void* stream);

/* ------------------------------------------------------- algorithmic work
 * Work per unit of the similarity solve, the roofline's numerator: transcendental
 * calls (pow counted as one; sqrt and cbrt included) and other floating-point
 * operations, per iteration of the reference's fixed point (three similarity
 * profiles, six psi evaluations, q_s, gustiness, roughness) and per cell for the
 * prologue and the flux epilogue. A solve's work is the sum over its cells of
 * PROLOGUE + iterations * ITER + EPILOGUE, the iterations those of the FP64 cold
 * start (the reference's own count), so a warm start shows as a higher rate. */
#define NESF_WORK_ITER_TRANSCENDENTALS 55
#define NESF_WORK_ITER_FLOPS 300
#define NESF_WORK_PROLOGUE_TRANSCENDENTALS 2
#define NESF_WORK_PROLOGUE_FLOPS 20
#define NESF_WORK_EPILOGUE_TRANSCENDENTALS 1
#define NESF_WORK_EPILOGUE_FLOPS 35
/* bytes per solved cell with FP32 fields: 9 inputs and 9 outputs of 4 bytes */
#define NESF_WORK_BYTES_PER_CELL_F32 72

/* ---------------------------------------------------------------- tracing
 * Kernel-boundary timeline of the coupling step: with tracing on, each
 * nesf_coupling_step (or a graph captured from one) records a CUDA event at its
 * start and after each kernel on the stream that ran it. nesf_trace_read returns,
 * for the last step (or replay) the device has finished, each mark's name, its
 * stream (0 the caller's, then the others in order of first use) and its time in
 * ms since the start mark; up to NESF_TRACE_MAX marks. Tracing adds no host
 * synchronisation to the step; reading waits for the marks. */
#define NESF_TRACE_MAX 64
typedef struct {
    char name[32];
    int32_t stream;
    int32_t pad_;
    double t_ms;
} nesf_trace_entry;

int nesf_trace_enable(nesf_context* ctx, int32_t on);
int nesf_trace_read(nesf_context* ctx, nesf_trace_entry* entries, int32_t max, int32_t* count);

#ifdef __cplusplus
}
#endif

#endif /* NESF_H */
