/*
 * nesf_oracle.h -- CPU FP64 restatement of NumericalEarth.jl's interface-flux
 * path. TEST INFRASTRUCTURE ONLY: it is the checker for the CUDA library and
 * the timed CPU baseline; nothing in the product links it.
 *
 * Arrays are HOST pointers to FP64 data in the layout of include/nesf.h
 * (dtype must be NESF_F64). Parity status: the similarity-theory solve, the
 * sea-ice fluxes and the assembly follow the reference files cited in
 * nesf_oracle.c line by line; the Thermodynamics.jl, Oceananigans and
 * ClimaSeaIce functions they call are restated from those packages' published
 * formulas (the packages are not vendored with the reference), so parity is
 * pinned only by the reference's known-answer tests (zero flux, neutral
 * log law, gustiness identities, stability values, three-equation
 * properties), which tests/test_oracle_known_answers.py reproduces.
 */
#ifndef NESF_ORACLE_H
#define NESF_ORACLE_H

#include "../include/nesf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* thermodynamics (Thermodynamics.jl restatement) */
double oracle_saturation_vapor_pressure(const nesf_thermodynamics_parameters* th, double T, int32_t phase);
double oracle_air_density(const nesf_thermodynamics_parameters* th, double T, double p, double q);
double oracle_cp_m(const nesf_thermodynamics_parameters* th, double q);
double oracle_latent_heat_vapor(const nesf_thermodynamics_parameters* th, double T);
double oracle_latent_heat_sublim(const nesf_thermodynamics_parameters* th, double T);
double oracle_virtual_temperature(const nesf_thermodynamics_parameters* th, double T, double q);
double oracle_surface_specific_humidity(const nesf_interface_params* p, double pa, double Ts);
double oracle_pow_ten_thirds(double x);
double oracle_dry_layer_humidity(const nesf_interface_params* p, double Tin, double Tla, double S, double Ta,
                                 double pa, double qa, double us, double qst, double qprev);

/* similarity-theory building blocks */
double oracle_stability(const nesf_stability_function* psi, double zeta);
double oracle_neutral_drag(const nesf_coefficient_fluxes* c, double U);
int oracle_al_fluxes(const nesf_interface_params* p, const nesf_al_fields* f);
double oracle_vsgs2(const nesf_similarity_theory_fluxes* f, double ustar, double bstar, double hbl);
double oracle_momentum_roughness(const nesf_roughness_length* r, double ustar, double U, double Ts);
double oracle_scalar_roughness(const nesf_roughness_length* r, double lu, double ustar, double U, double Ts);
double oracle_buoyancy_scale(const nesf_interface_params* p, double theta_star, double q_star, double Ts, double qs);

/* three-equation interface conditions: returns T*, S*, q */
void oracle_solve_interface_conditions(const nesf_io_params* p, double To, double So, double Si, double h,
                                       double hc, double Tsi, double* Tb, double* Sb, double* q);

/* grid drivers (OpenMP over rows when built with -fopenmp) */
int oracle_ao_fluxes(const nesf_interface_params* p, const nesf_ao_fields* f);
int oracle_ai_fluxes(const nesf_interface_params* p, const nesf_ai_fields* f);
int oracle_io_fluxes(const nesf_io_params* p, const nesf_io_fields* f);
int oracle_fractional_indices(const nesf_grid* g, const nesf_exchange_coords* c, const nesf_atmos_grid* a,
                              double* fi, double* fj);
int oracle_interpolate_atmosphere(const nesf_interp_fields* f);
int oracle_assemble_net_ocean_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f);
int oracle_assemble_net_sea_ice_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f);
int oracle_apply_air_sea_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f);
int oracle_apply_air_sea_ice_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f);
int oracle_assemble_net_land_fluxes(const nesf_land_flux_fields* f);
int oracle_apply_air_land_radiative_fluxes(const nesf_land_radiation_params* p, const nesf_land_flux_fields* f);

void oracle_set_threads(int32_t n);
void oracle_set_humidity_ulp_shift(int32_t n, int32_t carry);   /* conditioning probe for tests; 0 = off */
void oracle_set_temperature_ulp_shift(int32_t n);
void oracle_set_interface_temperature_ulp_shift(int32_t n);
int32_t oracle_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
