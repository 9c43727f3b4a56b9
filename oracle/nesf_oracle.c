/*
 * nesf_oracle.c -- CPU FP64 restatement of NumericalEarth.jl's interface-flux
 * path (reference: NumericalEarth.jl v0.6.2). TEST INFRASTRUCTURE ONLY: the
 * checker for the CUDA library and the timed CPU baseline.
 *
 * Every function cites the reference file:line it restates. Expressions keep
 * the reference's operation order (Julia evaluates left to right:
 * `a * b / c` is `(a * b) / c`). Functions of packages the reference calls but
 * does not vendor are restated from their published definitions:
 *   - Thermodynamics.jl (compat "0.15.3, 1"): saturation vapour pressure by the
 *     Clausius-Clapeyron integral with a linear latent heat, gas constant and
 *     heat capacity of moist air, latent heats, virtual temperature;
 *   - Oceananigans.jl (compat "0.110.15, 0.111"): two-point face/centre
 *     averages, fractional indices on a regular longitude-latitude grid,
 *     bilinear-in-space and linear-in-time interpolation;
 *   - ClimaSeaIce.jl (compat "0.5, 0.6"): LinearLiquidus melting temperature
 *     T_m = T_fw - slope * S.
 * Pinning: the reference is Julia and cannot run here, and its tests hold no
 * golden flux vectors. This restatement is pinned by the known answers those
 * tests do hold (zero fluxes, the neutral log-law closed form, gustiness bit
 * identity, Large-Yeager stability values, the three-equation interface
 * properties, the dry-layer and slab-land cases, e_sat at the triple point).
 * Parity unpinned: the restated Thermodynamics.jl, Oceananigans.jl and
 * ClimaSeaIce.jl functions above beyond those identities.
 * Build with -ffp-contract=off so that no fused multiply-add changes the
 * rounding between machines.
 */
#include "nesf_oracle.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void oracle_set_threads(int32_t n) { g_threads = n; }

/* Conditioning probe for the parity tests: each iterate's interface humidity is moved by n
 * units in the last place (0 = the reference's arithmetic), either only where the flux
 * evaluation sees it (carry = 0) or also in the iterate handed on (carry = 1). Where q_s - q_a
 * cancels, the reference's vapor fluxes respond to a last-place change of q_s (of any of its
 * ingredients) by ulp(q_a) / |q_s - q_a|, and the fixed point feeds the change back with the
 * slope of the q_s map; the two forms measure the response without and with that feedback. */
static int32_t g_humidity_ulp_shift = 0, g_humidity_shift_carry = 0;
void oracle_set_humidity_ulp_shift(int32_t n, int32_t carry) {
    g_humidity_ulp_shift = n;
    g_humidity_shift_carry = carry;
}
/* The same probe on the air's potential temperature theta_a (surface_atmosphere_temperature,
 * its ulp differs between a CPU and a GPU that contracts its multiply-add): where theta_a - T_s
 * cancels, the sensible heat responds to it by ulp(theta_a) / |theta_a - T_s|. */
static int32_t g_theta_ulp_shift = 0;
void oracle_set_temperature_ulp_shift(int32_t n) { g_theta_ulp_shift = n; }
/* ... and on each iterate's interface temperature T_s (a skin temperature's balance is
 * rounded differently by a GPU that contracts its multiply-adds). */
static int32_t g_ts_ulp_shift = 0;
void oracle_set_interface_temperature_ulp_shift(int32_t n) { g_ts_ulp_shift = n; }
int32_t oracle_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------ layout */
static inline int64_t idx2(const nesf_grid* g, int i, int j) {
    /* Oceananigans parent-array offset of (i, j), 1-based interior index */
    return (int64_t)(i - 1 + g->hx) + (int64_t)(j - 1 + g->hy) * g->stride_j;
}
static inline double rd(const void* a, int64_t k) { return ((const double*)a)[k]; }

/* Julia's min / max / clamp on floats: a NaN argument gives NaN (C's fmin/fmax
 * would drop it), and min(-0.0, 0.0) = -0.0, max(-0.0, 0.0) = 0.0. */
static inline double jmin(double x, double y) {
    if (isnan(x) || isnan(y)) return x + y;
    if (x == y) return signbit(x) ? x : y;
    return x < y ? x : y;
}
static inline double jmax(double x, double y) {
    if (isnan(x) || isnan(y)) return x + y;
    if (x == y) return signbit(x) ? y : x;
    return x > y ? x : y;
}
static inline double rdz(const void* a, int64_t k) { return a ? ((const double*)a)[k] : 0.0; }
static inline void wr(void* a, int64_t k, double v) { if (a) ((double*)a)[k] = v; }

/* ------------------------------------------------------ thermodynamics
 * Parameter accessors: src/Atmospheres/thermodynamic_parameters.jl:73-78,238-258 */
static inline double R_d(const nesf_thermodynamics_parameters* t) { return t->gas_constant / t->dry_air_molar_mass; }
static inline double R_v(const nesf_thermodynamics_parameters* t) { return t->gas_constant / t->water_molar_mass; }
static inline double Rv_over_Rd(const nesf_thermodynamics_parameters* t) { return t->dry_air_molar_mass / t->water_molar_mass; }
static inline double cp_d(const nesf_thermodynamics_parameters* t) { return R_d(t) / t->dry_air_adiabatic_exponent; }

/* Thermodynamics.jl saturation_vapor_pressure(param_set, T, phase):
 * p_tr (T/T_tr)^(dcp/R_v) exp[(L0 - dcp T0)/R_v (1/T_tr - 1/T)], dcp = cp_v - cp_{l|i}
 * (formula also in docs/src/interface_fluxes.md:86-97). */
double oracle_saturation_vapor_pressure(const nesf_thermodynamics_parameters* t, double T, int32_t phase) {
    double LH0 = phase == NESF_PHASE_ICE ? t->reference_sublimation_enthalpy : t->reference_vaporization_enthalpy;
    double cpc = phase == NESF_PHASE_ICE ? t->water_ice_heat_capacity : t->liquid_water_heat_capacity;
    double dcp = t->water_vapor_heat_capacity - cpc;
    double Rv = R_v(t);
    double Ttr = t->triple_point_temperature;
    double T0 = t->reference_temperature;
    return t->triple_point_pressure * pow(T / Ttr, dcp / Rv) * exp((LH0 - dcp * T0) / Rv * (1 / Ttr - 1 / T));
}

/* gas_constant_air: R_d (1 + (Rv/Rd - 1) q) for vapour only */
static inline double gas_constant_air(const nesf_thermodynamics_parameters* t, double q) {
    return R_d(t) * (1 + (Rv_over_Rd(t) - 1) * q);
}

double oracle_air_density(const nesf_thermodynamics_parameters* t, double T, double p, double q) {
    return p / (gas_constant_air(t, q) * T);
}

double oracle_cp_m(const nesf_thermodynamics_parameters* t, double q) {
    return cp_d(t) + (t->water_vapor_heat_capacity - cp_d(t)) * q;
}

double oracle_latent_heat_vapor(const nesf_thermodynamics_parameters* t, double T) {
    return t->reference_vaporization_enthalpy +
           (t->water_vapor_heat_capacity - t->liquid_water_heat_capacity) * (T - t->reference_temperature);
}

double oracle_latent_heat_sublim(const nesf_thermodynamics_parameters* t, double T) {
    return t->reference_sublimation_enthalpy +
           (t->water_vapor_heat_capacity - t->water_ice_heat_capacity) * (T - t->reference_temperature);
}

double oracle_virtual_temperature(const nesf_thermodynamics_parameters* t, double T, double q) {
    return gas_constant_air(t, q) / R_d(t) * T;
}

/* surface_specific_humidity(::ImpureSaturationSpecificHumidity, ...)
 * src/EarthSystemModels/InterfaceComputations/interface_states.jl:46-47,55-74 */
double oracle_surface_specific_humidity(const nesf_interface_params* p, double pa, double Ts) {
    const nesf_thermodynamics_parameters* t = &p->thermo;
    double x = p->has_water_mole_fraction ? p->water_mole_fraction : 1.0;
    double pv = x * oracle_saturation_vapor_pressure(t, Ts, p->humidity_phase);
    double einv = 1 / Rv_over_Rd(t);
    pv = jmin(pv, 0.999 * pa);
    return einv * pv / (pa - (1 - einv) * pv);
}

/* surface_atmosphere_temperature (interface_states.jl:308-317) */
static inline double surface_atmosphere_temperature(const nesf_interface_params* p, double Ta, double qa) {
    double c = oracle_cp_m(&p->thermo, qa);
    return Ta + p->gravitational_acceleration * p->surface_layer_height / c;
}

/* ------------------------------------------------- stability functions */
static inline double zmin0(double z) { return jmin(0.0, z); }
static inline double zmax0(double z) { return jmax(0.0, z); }

/* EdsonMomentumStabilityFunction (similarity_theory_turbulent_fluxes.jl:501-532) */
static double psi_edson_momentum(const double* c, double z) {
    double zmax = c[0], Ap = c[1], Bp = c[2], Cp = c[3], Dp = c[4];
    double Am = c[5], Bm = c[6], Cm = c[7], Dm = c[8], Em = c[9], Fm = c[10];
    double zm = zmin0(z), zp = zmax0(z);
    double dz = jmin(zmax, Ap * zp);
    double psip = -Bp * zp - Cp * (zp - Dp) * exp(-dz) - Cp * Dp;
    double f1 = sqrt(sqrt(1 - Am * zm));
    double psi1 = Bm * log((1 + f1) / Bm) + log((1 + f1 * f1) / Bm) - Bm * atan(f1) + Cm;
    double f2 = cbrt(1 - Dm * zm);
    double psi2 = Em / 2 * log((1 + f2 + f2 * f2) / Em) - sqrt(Em) * atan((1 + 2 * f2) / sqrt(Em)) + Fm;
    double f = zm * zm / (1 + zm * zm);
    double psim = (1 - f) * psi1 + f * psi2;
    return z < 0 ? psim : psip;
}

/* EdsonScalarStabilityFunction (similarity_theory_turbulent_fluxes.jl:586-618) */
static double psi_edson_scalar(const double* c, double z) {
    double zmax = c[0], Ap = c[1], Bp = c[2], Cp = c[3], Dp = c[4], Ep = c[5];
    double Am = c[6], Bm = c[7], Cm = c[8], Dm = c[9], Em = c[10], Fm = c[11];
    double zm = zmin0(z), zp = zmax0(z);
    double dz = jmin(zmax, Ap * zp);
    double psip = -pow(1 + Bp * zp, Cp) - Bp * (zp - Dp) * exp(-dz) - Ep;
    double f1 = sqrt(1 - Am * zm);
    double psi1 = Bm * log((1 + f1) / Bm) + Cm;
    double f2 = cbrt(1 - Dm * zm);
    double psi2 = Em / 2 * log((1 + f2 + f2 * f2) / Em) - sqrt(Em) * atan((1 + 2 * f2) / sqrt(Em)) + Fm;
    double f = zm * zm / (1 + zm * zm);
    double psim = (1 - f) * psi1 + f * psi2;
    return z < 0 ? psim : psip;
}

/* ShebaMomentumStabilityFunction (similarity_theory_turbulent_fluxes.jl:643-657) */
static double psi_sheba_momentum(double a, double b, double z) {
    double zp = zmax0(z);
    double x = cbrt(1 + zp);
    double B = cbrt((1 - b) / b);
    double rt3 = sqrt(3.0);
    double P1 = -3 * a * (x - 1) / b;
    double P2 = a * B / (2 * b) * (2 * log((x + B) / (1 + B)) - log((x * x - B * x + B * B) / (1 - B + B * B)) +
                                   2 * rt3 * (atan((2 * x - B) / (rt3 * B)) - atan((2 - B) / (rt3 * B))));
    return P1 + P2;
}

/* ShebaScalarStabilityFunction (similarity_theory_turbulent_fluxes.jl:665-677) */
static double psi_sheba_scalar(double a, double b, double c, double z) {
    double B = sqrt(c * c - 4);
    double zp = zmax0(z);
    double P1 = -b / 2 * log(1 + c * zp + zp * zp);
    double P2 = (b * c / (2 * B) - a / B) * (log((2 * zp + c - B) / (2 * zp + c + B)) - log((c - B) / (c + B)));
    return P1 + P2;
}

/* PaulsonMomentumStabilityFunction (similarity_theory_turbulent_fluxes.jl:688-699) */
static double psi_paulson_momentum(double a, double b, double z) {
    double zm = zmin0(z);
    double x = sqrt(sqrt(1 - a * zm));
    double P1 = 2 * log((1 + x) / 2);
    double P2 = log((1 + x * x) / 2);
    double P3 = -2 * atan(x);
    return P1 + P2 + P3 + b;
}

/* PaulsonScalarStabilityFunction (similarity_theory_turbulent_fluxes.jl:705-710) */
static double psi_paulson_scalar(double a, double z) {
    double zm = zmin0(z);
    double x = sqrt(sqrt(1 - a * zm));
    return 2 * log((1 + x * x) / 2);
}

/* LinearStableStabilityFunction (similarity_theory_turbulent_fluxes.jl:747-752) */
static double psi_linear(double coef, double zmax, double z) {
    double zp = zmax0(z);
    return -coef * jmin(zp, zmax);
}

/* stability_profile dispatch; SplitStabilityFunction (:720-725) selects stable for z > 0 */
double oracle_stability(const nesf_stability_function* s, double z) {
    const double* c = s->c;
    switch (s->kind) {
    case NESF_PSI_ZERO: return 0.0;
    case NESF_PSI_EDSON_MOMENTUM: return psi_edson_momentum(c, z);
    case NESF_PSI_EDSON_SCALAR: return psi_edson_scalar(c, z);
    case NESF_PSI_SHEBA_PAULSON_MOMENTUM: {
        double st = psi_sheba_momentum(c[0], c[1], z);
        double un = psi_paulson_momentum(c[2], c[3], z);
        return z > 0 ? st : un;
    }
    case NESF_PSI_SHEBA_PAULSON_SCALAR: {
        double st = psi_sheba_scalar(c[0], c[1], c[2], z);
        double un = psi_paulson_scalar(c[3], z);
        return z > 0 ? st : un;
    }
    case NESF_PSI_LINEAR_PAULSON_MOMENTUM: {
        double st = psi_linear(c[0], c[1], z);
        double un = psi_paulson_momentum(c[2], c[3], z);
        return z > 0 ? st : un;
    }
    case NESF_PSI_LINEAR_PAULSON_SCALAR: {
        double st = psi_linear(c[0], c[1], z);
        double un = psi_paulson_scalar(c[2], z);
        return z > 0 ? st : un;
    }
    default: return NAN;
    }
}

/* similarity_profile (similarity_theory_turbulent_fluxes.jl:242-253) */
static double similarity_profile(int form, const nesf_stability_function* psi, double h, double l, double L) {
    double zeta = h / L;
    double ph = oracle_stability(psi, zeta);
    if (form == NESF_PROFILE_COARE) return log(h / l) - ph;
    double pl = oracle_stability(psi, l / L);
    return log(h / l) - ph + pl;
}

/* vsgs2 (similarity_theory_turbulent_fluxes.jl:88-98): convective + mesoscale slots */
double oracle_vsgs2(const nesf_similarity_theory_fluxes* f, double ustar, double bstar, double hbl) {
    double conv = 0.0;
    if (f->subgrid_kind == NESF_SUBGRID_CONSTANT) {
        conv = f->constant_subgrid_velocity * f->constant_subgrid_velocity;
    } else if (f->subgrid_kind == NESF_SUBGRID_CONVECTIVE) {
        double Jb = -ustar * bstar;
        double UG = jmax(f->minimum_gustiness, f->gustiness_parameter * cbrt(jmax(0.0, Jb) * hbl));
        conv = UG * UG;
    }
    double meso = f->mesoscale_subgrid_velocity * f->mesoscale_subgrid_velocity;
    return conv + meso;
}

/* compute_air_kinematic_viscosity (roughness_lengths.jl:182-189) */
static double air_viscosity(const nesf_roughness_length* r, double T) {
    if (r->viscosity_kind == 0) return r->air_kinematic_viscosity;
    const double* C = r->viscosity_coefficients;
    double Tc = T - 273.15;
    return C[0] + C[1] * Tc + C[2] * Tc * Tc + C[3] * (Tc * Tc * Tc);
}

/* roughness_length(::MomentumRoughnessLength) (roughness_lengths.jl:74-75,197-210) */
double oracle_momentum_roughness(const nesf_roughness_length* r, double ustar, double U, double Ts) {
    if (r->kind == NESF_ROUGHNESS_CONSTANT) return r->value;
    double nu = air_viscosity(r, Ts);
    double g = r->gravitational_acceleration;
    double Cg = r->charnock;
    if (r->wave_kind == 1) Cg = jmax(0.0, r->wave_c1 * jmin(U, r->wave_umax) + r->wave_c2);
    double Cnu = r->smooth_wall_parameter;
    double lW = Cg * (ustar * ustar) / g;
    double lR = Cnu == 0 ? 0.0 : Cnu * nu / ustar;
    double ls = lW + lR;
    return jmin(ls, r->maximum_roughness_length);
}

/* roughness_length(::ScalarRoughnessLength) + ReynoldsScalingFunction (roughness_lengths.jl:231-246) */
double oracle_scalar_roughness(const nesf_roughness_length* r, double lu, double ustar, double U, double Ts) {
    (void)U;
    if (r->kind == NESF_ROUGHNESS_CONSTANT) return r->value;
    double nu = air_viscosity(r, Ts);
    double Rs = lu * ustar / nu;
    double ls = Rs == 0 ? 0.0 : r->reynolds_A / pow(Rs, r->reynolds_b);
    return jmin(ls, r->maximum_roughness_length);
}

/* buoyancy_scale (similarity_theory_turbulent_fluxes.jl:417-425) */
double oracle_buoyancy_scale(const nesf_interface_params* p, double th, double qst, double Ts, double qs) {
    double Tv = oracle_virtual_temperature(&p->thermo, Ts, qs);
    double eps = Rv_over_Rd(&p->thermo);
    double delta = eps - 1;
    return p->gravitational_acceleration / Tv * (th * (1 + delta * qs) + delta * Tv * qst);
}

/* ----------------------------------------------------- the fixed point */
typedef struct {
    double ua, va, Ta, pa, qa;       /* atmosphere state                  */
    double ui, vi;                   /* interface velocities              */
    double Ti, Si;                   /* interior temperature (K), salinity */
    double hi, hs, hc;               /* ice state (skin over ice)         */
    double sw, lw;                   /* downwelling radiation             */
    double kappa;                    /* interior diffusivity              */
    double sat;                      /* land surface saturation           */
} cell_in;

typedef struct { double us, ts, qs_, T, q; } istate;  /* u*, theta*, q*, T_s, q_s */

/* iterate_interface_fluxes (similarity_theory_turbulent_fluxes.jl:315-385) */
static void iterate_fluxes(const nesf_interface_params* p, const cell_in* c, double Ts, double qs, double dth,
                           double dq, double dh, const istate* prev, double* us, double* ts, double* qst) {
    const nesf_similarity_theory_fluxes* F = &p->fluxes;
    double ustar = prev->us, tstar = prev->ts, qstar = prev->qs_;
    double bstar = oracle_buoyancy_scale(p, tstar, qstar, Ts, qs);
    double Usg2 = oracle_vsgs2(F, ustar, bstar, p->boundary_layer_height);
    double du, dv;
    if (p->velocity_formulation == NESF_WIND_VELOCITY) { du = c->ua; dv = c->va; }
    else { du = c->ua - c->ui; dv = c->va - c->vi; }
    double U = sqrt(du * du + dv * dv + Usg2);
    double lu = oracle_momentum_roughness(&F->roughness[0], ustar, U, Ts);
    double lq = oracle_scalar_roughness(&F->roughness[2], lu, ustar, U, Ts);
    double lt = oracle_scalar_roughness(&F->roughness[1], lu, ustar, U, Ts);
    double h = jmax(dh - F->zero_plane_displacement, 2 * lu);   /* displaced_profile_height (:313) */
    double k = F->von_karman_constant;
    double L = bstar == 0 ? INFINITY : ustar * ustar / (k * bstar);
    double chiu = k / similarity_profile(F->similarity_form, &F->stability[0], h, lu, L);
    double chit = k / similarity_profile(F->similarity_form, &F->stability[1], h, lt, L);
    double chiq = k / similarity_profile(F->similarity_form, &F->stability[2], h, lq, L);
    *us = chiu * U;
    *ts = chit * dth;
    *qst = chiq * dq;
}

/* PolynomialNeutralDragCoefficient (coefficient_based_turbulent_fluxes.jl:48-54) */
double oracle_neutral_drag(const nesf_coefficient_fluxes* c, double U) {
    U = jmax(U, c->minimum_wind_speed);
    double U6 = pow(U, 6);
    return U < c->high_wind_speed_threshold ? (c->drag_a / U + c->drag_b + c->drag_c * U - c->drag_d * U6) / 1000
                                            : c->high_wind_drag_coefficient;
}

/* iterate_interface_fluxes(::CoefficientBasedFluxes) (coefficient_based_turbulent_fluxes.jl:346-371)
 * with evaluate_coefficients: constants (:269-285) or Large-Yeager (:288-340) */
static void iterate_coefficient_fluxes(const nesf_interface_params* p, const cell_in* c, double Ts, double qs,
                                       double dth, double dq, double dh, const istate* prev, double* us,
                                       double* ts, double* qst) {
    const nesf_coefficient_fluxes* C = &p->coefficients;
    int ly = C->kind == NESF_COEFFICIENTS_LARGE_YEAGER;
    double du, dv;
    if (p->velocity_formulation == NESF_WIND_VELOCITY) { du = c->ua; dv = c->va; }
    else { du = c->ua - c->ui; dv = c->va - c->vi; }
    double Umin = ly ? C->minimum_wind_speed : 0.0;                    /* minimum_wind_speed (:265-267) */
    double dU = jmax(sqrt(du * du + dv * dv), Umin);
    double Cd = C->momentum, Ch = C->temperature, Cq = C->water_vapor;
    if (!ly && (C->polynomial_mask & 7)) {   /* evaluate_coefficient(::PolynomialNeutralDragCoefficient, dU) (:271) */
        double Cp = oracle_neutral_drag(C, dU);
        if (C->polynomial_mask & 1) Cd = Cp;
        if (C->polynomial_mask & 2) Ch = Cp;
        if (C->polynomial_mask & 4) Cq = Cp;
    }
    if (ly) {
        double k = C->von_karman_constant;
        double ustar = prev->us;
        dU = jmax(dU, C->minimum_wind_speed);                           /* :305 */
        double bstar = oracle_buoyancy_scale(p, prev->ts, prev->qs_, Ts, qs);
        double L = bstar == 0 ? INFINITY : ustar * ustar / (k * bstar);
        double zeta = dh / L;
        double psim = oracle_stability(&C->stability[0], zeta);
        double psih = oracle_stability(&C->stability[1], zeta);
        double Cdp = ustar == 0 ? oracle_neutral_drag(C, dU) : ustar * ustar / (dU * dU);
        double UN10 = dU / (1 + sqrt(Cdp) / k * (log(dh / C->reference_height) - psim));
        UN10 = jmax(UN10, C->minimum_wind_speed);
        double CdN = oracle_neutral_drag(C, UN10);
        int stable = zeta > 0;
        double ChN = sqrt(CdN) / 1000 * (stable ? C->stable_heat_transfer_coefficient
                                                : C->unstable_heat_transfer_coefficient);
        double CqN = sqrt(CdN) / 1000 * C->moisture_transfer_coefficient;
        double xim = sqrt(CdN) / k * (log(dh / C->reference_height) - psim);
        Cd = CdN / ((1 + xim) * (1 + xim));
        double xih = sqrt(CdN) / k * (log(dh / C->reference_height) - psih);
        double ratio = sqrt(Cd) / sqrt(CdN);
        Ch = ChN * ratio / (1 + ChN * xih);
        Cq = CqN * ratio / (1 + CqN * xih);
    }
    *us = sqrt(Cd) * dU;
    *ts = Cd == 0 ? 0.0 : Ch / sqrt(Cd) * dth;
    *qst = Cd == 0 ? 0.0 : Cq / sqrt(Cd) * dq;
}

/* Julia clamp: ifelse(x > hi, hi, ifelse(x < lo, lo, x)) (a NaN x stays NaN) */
static inline double clampd(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

/* compute_interface_temperature (interface_states.jl:333 bulk; 526-577 skin) with
 * flux_balance_temperature (434-457 diffusive; 468-524 conductive ice/snow) */
static double interface_temperature(const nesf_interface_params* p, const cell_in* c, const istate* s) {
    if (p->temperature_formulation == NESF_BULK_TEMPERATURE) return s->T;
    const nesf_thermodynamics_parameters* t = &p->thermo;
    double rho = oracle_air_density(t, c->Ta, c->pa, c->qa);
    double ca = oracle_cp_m(t, c->qa);
    double Li = oracle_latent_heat_sublim(t, c->Ta);
    double Tm1 = s->T;
    double sigma = p->has_radiation ? p->stefan_boltzmann_constant : 0.0;
    double eps = p->has_radiation ? p->emissivity : 0.0;
    double alb = p->has_radiation ? p->albedo : 0.0;
    double SW = p->has_radiation ? c->sw : 0.0;
    double LW = p->has_radiation ? c->lw : 0.0;
    double T2 = Tm1 * Tm1;
    double Iup = sigma * eps * (T2 * T2);
    double Qd = -(1 - alb) * SW - eps * LW;
    double QT = -rho * ca * s->us * s->ts;
    double Qv = -rho * Li * s->us * s->qs_;
    double Tat = surface_atmosphere_temperature(p, c->Ta, c->qa);
    if (p->temperature_formulation == NESF_SKIN_TEMPERATURE_DIFFUSIVE) {
        /* internal_diffusivity: a constant, or max(interior kappa, minimum) (interface_states.jl:390-391) */
        double kap = c->kappa >= 0 ? jmax(c->kappa, p->diffusive_kappa) : p->diffusive_kappa;
        double del = p->diffusive_delta;
        double rho_i = p->interior_reference_density, c_i = p->interior_heat_capacity;
        double Qa = Qv + Iup + Qd;
        double lam = 1 / (rho_i * c_i);
        double JT = Qa * lam;
        double dT = Tat - s->T;
        double OmT = QT * lam;
        double D = kap * dT - OmT * del;
        double Tst = (c->Ti * kap * dT - (JT * dT + OmT * Tat) * del) / D;
        Tst = D == 0 ? s->T : Tst;
        return c->Ti + clampd(Tst - c->Ti, -p->max_delta_T, p->max_delta_T);
    }
    /* conductive_flux_balance_temperature: R = h_s/k_s + h_i/k_i (or h_i/k_i bare ice) */
    double R = p->snow_conductivity > 0 ? c->hs / p->snow_conductivity + c->hi / p->ice_conductivity
                                        : c->hi / p->ice_conductivity;
    double off = p->interface_temperature_offset;   /* sea-ice temperature units */
    double Tb = p->liquidus_freshwater_melting_temperature - p->liquidus_slope * c->Si;
    Tb = Tb + off;
    double dT = Tat - Tm1;
    double Qa = Qv + Iup + Qd;
    double Om = dT == 0 ? 0.0 : QT / dT;
    double beta = 4 * Iup / Tm1;
    double D = 1 + beta * R - Om * R;
    double Tst = (Tb + beta * R * Tm1 - Om * R * Tat - Qa * R) / D;
    Tst = D == 0 ? Tm1 : Tst;
    Tst = isnan(Tst) ? Tm1 : Tst;
    double dTs = Tst - Tm1;
    double Tp = Tm1 + clampd(dTs, -p->max_delta_T, p->max_delta_T);
    double Tm = p->liquidus_freshwater_melting_temperature + off;
    Tp = jmin(Tp, Tm);
    Tp = c->hi >= c->hc ? Tp : Tb;
    return Tp;
}

/* theta^(10/3) (the Millington-Quirk power, dry_layer_humidity.jl:262), correctly rounded: the
 * exponent is 10/3 rounded to double, p = 10/3 + d with d = 2^-51 / 3, so
 * x^p = x^3 cbrt(x) x^d, with x^3 an exact double-double (Dekker products through fma), cbrt(x)
 * refined to double-double by one Newton step on c^3 = x, and x^d = 1 + d ln x to 1e-32. The
 * fixed point amplifies a last-place change of this power a thousandfold where the vapor
 * balance cancels, so the power is rounded once from a near-exact value rather than taken from
 * a libm pow (within about half an ulp, and misrounded in some cases). */
double oracle_pow_ten_thirds(double x) {
    if (!(x > 0x1p-300) || !(x < 0x1p300)) return pow(x, 10.0 / 3.0);
    double x2 = x * x, x2l = fma(x, x, -x2);
    double x3 = x2 * x, x3l = fma(x2, x, -x3) + x2l * x;
    double c = cbrt(x);
    double c2 = c * c, c2l = fma(c, c, -c2);
    double c3 = c2 * c, c3l = fma(c2, c, -c3) + c2l * c;
    double cl = -((c3 - x) + c3l) / (3.0 * c2);
    double ph = x3 * c;
    double pl = fma(x3, c, -ph) + (x3 * cl + x3l * c);
    pl += ph * ((0x1p-51 / 3.0) * log(x));
    return ph + pl;
}

/* DryLayerHumidity's compute_interface_humidity (dry_layer_humidity.jl:317-366) with
 * StorageBasedDryLayerDepth (:95-100) and the tortuosity models (:252-263). The dry layer's
 * depth follows the land saturation S; vapor leaves the front (saturated at
 * Te = Tin + chi (Tla - Tin)) by a Fick flux of conductance Ge and the atmosphere carries it
 * away at the previous iterate's flux Ja = -rho u* q*, linearised about q_prev; the series
 * solution is blended with the saturated skin q_sat(Tin) by a logistic weight in the depth.
 * Tin is the current interface-temperature iterate, Tla the bulk land temperature. */
double oracle_dry_layer_humidity(const nesf_interface_params* p, double Tin, double Tla, double S, double Ta,
                                 double pa, double qa, double us, double qst, double qprev) {
    double rho = oracle_air_density(&p->thermo, Ta, pa, qa);
    double s = jmin(S / p->dry_layer_onset_saturation, 1.0);
    double delta = p->maximum_dry_layer_depth * pow(jmax(1.0 - s, 0.0), p->dry_layer_exponent);
    double dmin = p->minimum_dry_layer_depth;
    double chi = clampd(delta / p->thermal_exchange_depth, 0.0, 1.0);
    double Te = Tin + chi * (Tla - Tin);
    double qe = oracle_surface_specific_humidity(p, pa, Te);
    double theta_l = S * p->porosity;                 /* pore liquid fraction ~ S nu */
    double Dv = p->molecular_diffusivity;             /* ConstantTortuosity */
    if (p->tortuosity == NESF_TORTUOSITY_POWER_LAW) { /* Millington-Quirk */
        double theta_g = jmax(p->porosity - theta_l, 0.0);
        Dv = p->molecular_diffusivity * oracle_pow_ten_thirds(theta_g) / (p->porosity * p->porosity);
    }
    double Ge = rho * Dv / jmax(delta, dmin);
    double Ja = -rho * us * qst;
    double dq = qprev - qa;
    double D = Ge * dq + Ja;
    double qseries = D == 0 ? qprev : (Ge * qe * dq + Ja * qa) / D;
    double qwet = oracle_surface_specific_humidity(p, pa, Tin);
    double w = p->wet_transition_width;
    double z = 10 * (delta - dmin - w / 2) / jmax(w, DBL_EPSILON);
    double sigma = 1 / (1 + exp(-z));
    return qwet + sigma * (qseries - qwet);
}

/* compute_interface_humidity (interface_states.jl:587-651): ImpureSaturationSpecificHumidity;
 * BulkHumidity (:120-125); FractionalHumidity with a constant beta or CriticalSaturation
 * (:152-158, 592-598); SkinHumidity's vapor-flux balance with the previous iterate (:626-651);
 * DryLayerHumidity (oracle_dry_layer_humidity).
 * saturation_specific_humidity (:76-90) is surface_specific_humidity with x = 1. */
static double interface_humidity(const nesf_interface_params* p, const cell_in* c, double Ts, const istate* prev) {
    switch (p->humidity_formulation) {
    case NESF_HUMIDITY_BULK: {
        double qsat = oracle_surface_specific_humidity(p, c->pa, Ts);
        return c->sat > 0 ? qsat : 0.0;
    }
    case NESF_HUMIDITY_FRACTIONAL: {
        double beta = p->critical_saturation > 0 ? jmin(c->sat / p->critical_saturation, 1.0)
                                                 : p->evaporation_efficiency;
        double qsat = oracle_surface_specific_humidity(p, c->pa, Ts);
        return beta * qsat;
    }
    case NESF_HUMIDITY_SKIN: {
        double rho = oracle_air_density(&p->thermo, c->Ta, c->pa, c->qa);
        double Td = c->Ti;                           /* bulk land temperature at the saturation depth */
        double qsat = oracle_surface_specific_humidity(p, c->pa, Td);
        double g = p->skin_vapor_diffusivity / p->skin_surface_thickness;
        double Ja = -rho * prev->us * prev->qs_;
        double dq = prev->q - c->qa;
        double D = g * dq + Ja;
        double qs = (g * qsat * dq + Ja * c->qa) / D;
        return D == 0 ? prev->q : qs;
    }
    case NESF_HUMIDITY_DRY_LAYER:
        return oracle_dry_layer_humidity(p, Ts, c->Ti, c->sat, c->Ta, c->pa, c->qa, prev->us, prev->qs_, prev->q);
    default:
        return oracle_surface_specific_humidity(p, c->pa, Ts);
    }
}

/* iterate_interface_state (compute_interface_state.jl:69-122) */
static istate iterate_state(const nesf_interface_params* p, const cell_in* c, const istate* prev) {
    double Ts = interface_temperature(p, c, prev);
    for (int32_t k = 0; k < g_ts_ulp_shift; k++) Ts = nextafter(Ts, INFINITY);
    double q_iter = interface_humidity(p, c, Ts, prev);
    double qs = q_iter;
    for (int32_t k = 0; k < g_humidity_ulp_shift; k++) qs = nextafter(qs, INFINITY);
    if (g_humidity_shift_carry) q_iter = qs;
    double dq = c->qa - qs;
    double tha = surface_atmosphere_temperature(p, c->Ta, c->qa);
    for (int32_t k = 0; k < g_theta_ulp_shift; k++) tha = nextafter(tha, INFINITY);
    double dth = tha - Ts;
    double dh = p->surface_layer_height;
    istate n;
    if (p->flux_formulation == NESF_FLUXES_COEFFICIENT_BASED)
        iterate_coefficient_fluxes(p, c, Ts, qs, dth, dq, dh, prev, &n.us, &n.ts, &n.qs_);
    else
        iterate_fluxes(p, c, Ts, qs, dth, dq, dh, prev, &n.us, &n.ts, &n.qs_);
    n.T = Ts;
    n.q = q_iter;
    return n;
}

/* the flux formulation's solver_stop_criteria kind */
static int stop_kind_of(const nesf_interface_params* p) {
    return p->flux_formulation == NESF_FLUXES_COEFFICIENT_BASED ? p->coefficients.stop_kind : p->fluxes.stop_kind;
}

/* iterating + compute_interface_state (compute_interface_state.jl:10-24,31-58) */
static istate solve(const nesf_interface_params* p, const cell_in* c, istate s0, int* iters) {
    /* the flux formulation's solver_stop_criteria */
    const int coef = p->flux_formulation == NESF_FLUXES_COEFFICIENT_BASED;
    const int stop_kind = coef ? p->coefficients.stop_kind : p->fluxes.stop_kind;
    const int maxiter = coef ? p->coefficients.maxiter : p->fluxes.maxiter;
    const double tolerance = coef ? p->coefficients.tolerance : p->fluxes.tolerance;
    istate sn = s0, sm = s0;
    int it = 0;
    for (;;) {
        int go;
        if (stop_kind == NESF_STOP_FIXED_ITERATIONS) {
            go = it < maxiter;
        } else {
            int hasnt_started = it == 0;
            int reached = it >= maxiter;
            double drift = fabs(sn.us - sm.us) + fabs(sn.ts - sm.ts) + fabs(sn.qs_ - sm.qs_);
            int converged = drift < tolerance;
            go = (!(converged | reached)) | hasnt_started;
        }
        if (!go) break;
        sm = sn;
        sn = iterate_state(p, c, &sm);
        it++;
    }
    *iters = it;
    return sn;
}

/* ---------------------------------------------------------- AO driver
 * _compute_atmosphere_ocean_interface_state! (atmosphere_ocean_fluxes.jl:62-71,80-197),
 * launched over (0:nx+1, 0:ny+1) (InterfaceComputations.jl:100-116). */
int oracle_ao_fluxes(const nesf_interface_params* p, const nesf_ao_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    if (g->hx < 2 || g->hy < 2) return NESF_ERR_ARG;
    const nesf_thermodynamics_parameters* t = &p->thermo;
    int nth = oracle_get_threads();
    (void)nth;
#pragma omp parallel for collapse(2) schedule(dynamic, 128) num_threads(nth)
    for (int j = 0; j <= g->ny + 1; j++) {
        for (int i = 0; i <= g->nx + 1; i++) {
            int64_t k = idx2(g, i, j);
            cell_in c;
            c.ua = rd(f->u_atm, k); c.va = rd(f->v_atm, k); c.Ta = rd(f->T_atm, k);
            c.pa = rd(f->p_atm, k); c.qa = rd(f->q_atm, k);
            /* assemble_interior_state: centre averages of the face velocities */
            c.ui = (rd(f->u_oc, k) + rd(f->u_oc, idx2(g, i + 1, j))) / 2;
            c.vi = (rd(f->v_oc, k) + rd(f->v_oc, idx2(g, i, j + 1))) / 2;
            c.Ti = rd(f->T_oc, k) + p->interior_temperature_offset;
            c.Si = rd(f->S_oc, k);
            c.hi = c.hs = c.hc = 0;
            c.sw = rdz(f->sw_down, k); c.lw = rdz(f->lw_down, k);
            c.kappa = f->kappa ? rd(f->kappa, k) : -1.0;
            int land = f->inactive ? f->inactive[k] != 0 : 0;

            double ustar0 = 1e-4;
            double qs0 = oracle_surface_specific_humidity(p, c.pa, c.Ti);
            istate s0 = {ustar0, ustar0, ustar0, c.Ti, qs0};
            istate s;
            int iters = 0;
            int needs_to_converge = stop_kind_of(p) == NESF_STOP_CONVERGENCE;
            double ui = c.ui, vi = c.vi;
            if (needs_to_converge && land) {
                istate z = {0, 0, 0, 273.15, 0};
                s = z;
            } else {
                s = solve(p, &c, s0, &iters);
            }
            if (land) {   /* zero_interface_state (interface_states.jl:800-803) */
                istate z = {0, 0, 0, 273.15, 0};
                s = z;
                ui = 0; vi = 0;
            }
            double us = s.us, ts = s.ts, qs = s.qs_;
            double du, dv;
            if (p->velocity_formulation == NESF_WIND_VELOCITY) { du = c.ua; dv = c.va; }
            else { du = c.ua - ui; dv = c.va - vi; }
            double dU = sqrt(du * du + dv * dv);
            double tx = dU == 0 ? 0.0 : -(us * us) * du / dU;
            double ty = dU == 0 ? 0.0 : -(us * us) * dv / dU;
            double rho = oracle_air_density(t, c.Ta, c.pa, c.qa);
            double cp = oracle_cp_m(t, c.qa);
            double Lv = oracle_latent_heat_vapor(t, c.Ta);
            wr(f->latent_heat, k, -rho * Lv * us * qs);
            wr(f->sensible_heat, k, -rho * cp * us * ts);
            wr(f->water_vapor, k, -rho * us * qs);
            wr(f->x_momentum, k, rho * tx);
            wr(f->y_momentum, k, rho * ty);
            wr(f->interface_temperature, k, s.T - p->interface_temperature_offset);
            wr(f->friction_velocity, k, us);
            wr(f->temperature_scale, k, ts);
            wr(f->water_vapor_scale, k, qs);
            if (f->iterations) f->iterations[k] = iters;
        }
    }
    return NESF_OK;
}

/* ---------------------------------------------------------- AI driver
 * _compute_atmosphere_sea_ice_interface_state! (atmosphere_sea_ice_fluxes.jl:65-185) */
/* ---------------------------------------------------------- AL driver
 * _compute_atmosphere_land_interface_state! (atmosphere_land_fluxes.jl:146-251), over the
 * interior (:89-102); T_s = the bulk land temperature (BulkTemperature), surface at rest. */
int oracle_al_fluxes(const nesf_interface_params* p, const nesf_al_fields* f) {
    if (f->dtype != NESF_F64) return 1;
    const nesf_grid* g = &f->grid;
    const nesf_thermodynamics_parameters* t = &p->thermo;
    int nth = oracle_get_threads();
#pragma omp parallel for collapse(2) schedule(dynamic, 128) num_threads(nth)
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j);
            cell_in c;
            memset(&c, 0, sizeof c);
            c.ua = rd(f->u_atm, k); c.va = rd(f->v_atm, k); c.Ta = rd(f->T_atm, k);
            c.pa = rd(f->p_atm, k); c.qa = rd(f->q_atm, k);
            c.ui = 0; c.vi = 0;
            c.Ti = rd(f->land_temperature, k);
            c.sat = f->saturation ? rd(f->saturation, k) : 1.0;
            c.kappa = -1.0;
            double ustar0 = 1e-4;
            double qs0 = oracle_surface_specific_humidity(p, c.pa, c.Ti);   /* :200-201 */
            istate s0 = {ustar0, ustar0, ustar0, c.Ti, qs0};
            int iters = 0;
            istate s = solve(p, &c, s0, &iters);
            double du = c.ua, dv = c.va;   /* velocity_difference with u_s = v_s = 0 */
            double dU = sqrt(du * du + dv * dv);
            double tx = dU == 0 ? 0.0 : -(s.us * s.us) * du / dU;
            double ty = dU == 0 ? 0.0 : -(s.us * s.us) * dv / dU;
            double rho = oracle_air_density(t, c.Ta, c.pa, c.qa);
            double cp = oracle_cp_m(t, c.qa);
            double Lv = oracle_latent_heat_vapor(t, c.Ta);
            wr(f->latent_heat, k, -rho * Lv * s.us * s.qs_);
            wr(f->sensible_heat, k, -rho * cp * s.us * s.ts);
            wr(f->water_vapor, k, -rho * s.us * s.qs_);
            wr(f->x_momentum, k, rho * tx);
            wr(f->y_momentum, k, rho * ty);
            wr(f->interface_temperature, k, s.T);
            wr(f->friction_velocity, k, s.us);
            wr(f->temperature_scale, k, s.ts);
            wr(f->water_vapor_scale, k, s.qs_);
            if (f->iterations) f->iterations[k] = iters;
        }
    }
    return 0;
}

int oracle_ai_fluxes(const nesf_interface_params* p, const nesf_ai_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    if (g->hx < 1 || g->hy < 1) return NESF_ERR_ARG;
    const nesf_thermodynamics_parameters* t = &p->thermo;
    int nth = oracle_get_threads();
    (void)nth;
#pragma omp parallel for collapse(2) schedule(dynamic, 128) num_threads(nth)
    for (int j = 0; j <= g->ny + 1; j++) {
        for (int i = 0; i <= g->nx + 1; i++) {
            int64_t k = idx2(g, i, j);
            cell_in c;
            c.ua = rd(f->u_atm, k); c.va = rd(f->v_atm, k); c.Ta = rd(f->T_atm, k);
            c.pa = rd(f->p_atm, k); c.qa = rd(f->q_atm, k);
            c.Ti = rd(f->T_oc, k) + p->interior_temperature_offset;
            c.Si = rd(f->S_oc, k);
            c.ui = 0; c.vi = 0;
            c.hi = rd(f->ice_thickness, k);
            c.hs = rdz(f->snow_thickness, k);
            c.hc = rd(f->consolidation_thickness, k);
            double aleph = rd(f->ice_concentration, k);
            double Ts0 = rd(f->interface_temperature, k) + p->interface_temperature_offset;
            c.sw = rdz(f->sw_down, k); c.lw = rdz(f->lw_down, k);
            c.kappa = -1.0;
            int land = f->inactive ? f->inactive[k] != 0 : 0;

            double ustar0 = 1e-4;
            double qs0 = oracle_surface_specific_humidity(p, c.pa, Ts0);
            istate s0 = {ustar0, ustar0, ustar0, Ts0, qs0};
            int ice_free = aleph == 0;
            int needs_to_converge = stop_kind_of(p) == NESF_STOP_CONVERGENCE;
            istate s;
            int iters = 0;
            if ((needs_to_converge && land) || ice_free) {
                istate z = {0, 0, 0, c.Ti, 0};
                s = z;
            } else {
                s = solve(p, &c, s0, &iters);
            }
            double us = s.us, ts = s.ts, qs = s.qs_;
            double du = c.ua - 0.0, dv = c.va - 0.0;
            if (p->velocity_formulation == NESF_WIND_VELOCITY) { du = c.ua; dv = c.va; }
            double dU = sqrt(du * du + dv * dv);
            double tx = dU == 0 ? 0.0 : -(us * us) * du / dU;
            double ty = dU == 0 ? 0.0 : -(us * us) * dv / dU;
            double rho = oracle_air_density(t, c.Ta, c.pa, c.qa);
            double cp = oracle_cp_m(t, c.qa);
            double Li = oracle_latent_heat_sublim(t, c.Ta);
            wr(f->latent_heat, k, -rho * us * qs * Li);
            wr(f->sensible_heat, k, -rho * cp * us * ts);
            wr(f->water_vapor, k, -rho * us * qs);
            wr(f->x_momentum, k, rho * tx);
            wr(f->y_momentum, k, rho * ty);
            ((double*)f->interface_temperature)[k] = s.T - p->interface_temperature_offset;
            if (f->iterations) f->iterations[k] = iters;
        }
    }
    return NESF_OK;
}

/* ------------------------------------------------------ sea-ice-ocean
 * solve_interface_conditions (sea_ice_ocean_heat_flux_formulations.jl:249-313) */
void oracle_solve_interface_conditions(const nesf_io_params* p, double To, double So, double Si, double h,
                                       double hc, double Tsi, double* Tb, double* Sb, double* q) {
    double E = p->reference_latent_heat;
    double kap = 0.0, Ti = 0.0;
    if (p->conductive) {
        int consolidated = h >= hc;
        kap = consolidated ? p->ice_conductivity / (h * E) : 0.0;
        Ti = Tsi;
    }
    double l1 = -p->liquidus_slope;
    double l2 = p->liquidus_freshwater_melting_temperature;
    double us = p->friction_velocity;
    double eta = p->ocean_reference_density * p->ocean_heat_capacity * p->heat_transfer_coefficient * us / E;
    double gam = p->ocean_reference_density * p->salt_transfer_coefficient * us;
    double th = eta + kap;
    double a = th * l1;
    double b = -gam - eta * To - kap * Ti + th * (l2 - l1 * Si);
    double c = gam * So + (eta * To + kap * Ti - th * l2) * Si;
    double xi = a == 0 ? 0.0 : 1 / (2 * a);
    double D = jmax(b * b - 4 * a * c, 0.0);
    double S = (-b - sqrt(D)) * xi;
    S = S < 0 ? (-b + sqrt(D)) * xi : S;
    double T = l2 - p->liquidus_slope * S;
    *Tb = T;
    *Sb = S;
    *q = eta * (To - T) + kap * (Ti - T);
}

/* _compute_sea_ice_ocean_fluxes! (sea_ice_ocean_fluxes.jl:106-226), interior launch (:xy).
 * Ocean temperature and salinity are 3-D (nz levels, stride_k); T is mutated by frazil. */
int oracle_io_fluxes(const nesf_io_params* p, const nesf_io_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    double rho = p->ocean_reference_density, cpo = p->ocean_heat_capacity;
    int nth = oracle_get_threads();
    (void)nth;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k2 = idx2(g, i, j);
            double* T = (double*)f->T_oc;
            const double* S = (const double*)f->S_oc;
            double dQ = 0.0;
            for (int kk = p->nz; kk >= 1; kk--) {
                int64_t k3 = k2 + (int64_t)(kk - 1) * p->stride_k;
                double dz = f->dz[kk - 1];
                double Tk = T[k3], Sk = S[k3];
                double Tm = p->liquidus_freshwater_melting_temperature - p->liquidus_slope * Sk;
                int freezing = Tk < Tm;
                double dE = (double)freezing * rho * cpo * (Tm - Tk);
                T[k3] = freezing ? Tm : Tk;
                dQ -= dE * dz / p->dt;
            }
            wr(f->frazil_heat, k2, dQ);
            int64_t kN = k2 + (int64_t)(p->nz - 1) * p->stride_k;
            double TN = T[kN], SN = S[kN];
            double Si = rd(f->ice_salinity, k2);
            double h = rd(f->ice_thickness, k2);
            double aleph = rd(f->ice_concentration, k2);
            double hc = rd(f->consolidation_thickness, k2);
            double Tsi = (p->conductive && f->internal_temperature) ? rd(f->internal_temperature, k2) : 0.0;
            double Qio, Tb, Sb;
            if (p->formulation == 1) {
                /* IceBathHeatFlux (sea_ice_ocean_heat_flux_formulations.jl:176-195) */
                double Tm = p->liquidus_freshwater_melting_temperature - p->liquidus_slope * SN;
                Qio = rho * cpo * p->heat_transfer_coefficient * p->friction_velocity * (TN - Tm) * aleph;
                Tb = Tm; Sb = SN;
            } else {
                double q;
                oracle_solve_interface_conditions(p, TN, SN, Si, h, hc, Tsi, &Tb, &Sb, &q);
                Qio = p->reference_latent_heat * q * aleph;
                wr(f->interface_T, k2, Tb);
                wr(f->interface_S, k2, Sb);
            }
            wr(f->interface_heat, k2, Qio);
            double Ei = rdz(f->ice_mass_flux, k2), Es = rdz(f->snow_mass_flux, k2);
            wr(f->freshwater, k2, -(Ei + Es) / rho);
            wr(f->salt, k2, Ei * Si / rho);
        }
    }
    return NESF_OK;
}

/* ---------------------------------------------------------- interpolation
 * _compute_fractional_indices! (prescribed_atmosphere_regridder.jl:51-71) with the
 * Oceananigans fractional index (x - x1)/dx + 1 on a regular longitude-latitude grid. */
int oracle_fractional_indices(const nesf_grid* g, const nesf_exchange_coords* c, const nesf_atmos_grid* a,
                              double* fi, double* fj) {
    for (int j = 1 - g->hy; j <= g->ny + g->hy; j++) {
        for (int i = 1 - g->hx; i <= g->nx + g->hx; i++) {
            int64_t k = idx2(g, i, j);
            double lon = c->lon0 + (i - 1) * c->dlon;
            double lat = c->lat0 + (j - 1) * c->dlat;
            fi[k] = (lon - a->lon0) / a->dlon + 1;
            fj[k] = (lat - a->lat0) / a->dlat + 1;
        }
    }
    return NESF_OK;
}

static inline int wrap_i(int i, int n) { int m = (i - 1) % n; if (m < 0) m += n; return m + 1; }
static inline int clamp_j(int j, int n) { return j < 1 ? 1 : (j > n ? n : j); }

/* interpolate(FractionalIndices, time, data): bilinear in (i, j), linear in time:
 * psi = psi2 * n + psi1 * (1 - n); periodic in longitude, clamped in latitude. */
static double interp_one(const nesf_atmos_grid* a, const double* d, double fi, double fj, double tn) {
    double fli = floor(fi), flj = floor(fj);
    int im = (int)fli, jm = (int)flj;
    double xi = fi - fli, eta = fj - flj;
    int i0 = wrap_i(im, a->nx), i1 = wrap_i(im + 1, a->nx);
    int j0 = clamp_j(jm, a->ny), j1 = clamp_j(jm + 1, a->ny);
    double v[2];
    for (int n = 0; n < 2; n++) {
        const double* b = d + (int64_t)n * a->stride_t;
#define AT(ii, jj) b[(int64_t)((ii) - 1 + a->hx) + (int64_t)((jj) - 1 + a->hy) * a->stride_j]
        v[n] = (1 - xi) * (1 - eta) * AT(i0, j0) + (1 - xi) * eta * AT(i0, j1) + xi * (1 - eta) * AT(i1, j0) +
               xi * eta * AT(i1, j1);
#undef AT
    }
    return v[1] * tn + v[0] * (1 - tn);
}

/* _interpolate_primary_atmospheric_state! (interpolate_atmospheric_state.jl:91-137) and
 * _interpolate_radiation_state! (interpolate_radiation_state.jl:43-69): halo ring launch.
 * intrinsic_vector is the identity on a longitude-latitude exchange grid. */
int oracle_interpolate_atmosphere(const nesf_interp_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    const nesf_atmos_grid* a = &f->atmos;
    for (int j = 0; j <= g->ny + 1; j++) {
        for (int i = 0; i <= g->nx + 1; i++) {
            int64_t k = idx2(g, i, j);
            double fi, fj;
            if (f->frac_i) { fi = f->frac_i[k]; fj = f->frac_j[k]; }
            else {
                double lon = f->coords.lon0 + (i - 1) * f->coords.dlon;
                double lat = f->coords.lat0 + (j - 1) * f->coords.dlat;
                fi = (lon - a->lon0) / a->dlon + 1;
                fj = (lat - a->lat0) / a->dlat + 1;
            }
            double tn = f->time_weight;
            const void* src[9] = {f->u, f->v, f->T, f->q, f->p, f->rain, f->snow, f->sw_down, f->lw_down};
            void* dst[9] = {f->u_out, f->v_out, f->T_out, f->q_out, f->p_out, f->rain_out, f->snow_out,
                            f->sw_out, f->lw_out};
            for (int n = 0; n < 9; n++) {
                if (!dst[n]) continue;
                double val = src[n] ? interp_one(a, (const double*)src[n], fi, fj, tn) : 0.0;
                ((double*)dst[n])[k] = val;
            }
        }
    }
    return NESF_OK;
}

/* ---------------------------------------------------------- assembly
 * _assemble_net_ocean_fluxes! (assemble_net_ocean_fluxes.jl:6,74-153); face values use the
 * two-point average (f[i-1] + f[i]) / 2 of Oceananigans' interpolation operators. */
int oracle_assemble_net_ocean_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    double rinv = 1 / p->ocean_reference_density;
    double cinv = 1 / p->ocean_heat_capacity;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j), kw = idx2(g, i - 1, j), ks = idx2(g, i, j - 1);
            double a = rdz(f->ice_concentration, k);
            double To = rd(f->ocean_surface_temperature, k);
            double Jr = rdz(f->rain, k), Js = rdz(f->snow, k), Ps = rdz(f->intercepted_snow, k);
            double Jl = rdz(f->land_freshwater, k);
            double QT = rd(f->ao_sensible, k), Qv = rd(f->ao_latent, k), Jv = rd(f->ao_water_vapor, k);
            double SQao = (QT + Qv) * (1 - a);
            double SFao = -(Jr + Jl + Js - Ps) * rinv + (1 - a) * Jv * rinv;
            double Jwao = -SFao;
            int inactive = f->inactive ? f->inactive[k] != 0 : 0;
            double Qin = rdz(f->io_interface_heat, k);
            double Jsio = rdz(f->io_salt, k);
            double Jwio = rdz(f->io_freshwater, k);
            double JTao = SQao * rinv * cinv;
            double JTio = Qin * rinv * cinv;
            double aw = rdz(f->ice_concentration, kw), as = rdz(f->ice_concentration, ks);
            double tcx = rinv * (1 - a) * rd(f->ao_x_momentum, k);
            double tcxw = rinv * (1 - aw) * rd(f->ao_x_momentum, kw);
            double tcy = rinv * (1 - a) * rd(f->ao_y_momentum, k);
            double tcys = rinv * (1 - as) * rd(f->ao_y_momentum, ks);
            double txao = (tcxw + tcx) / 2;
            double tyao = (tcys + tcy) / 2;
            double txio = rdz(f->io_x_momentum, k) * rinv * ((aw + a) / 2);
            double tyio = rdz(f->io_y_momentum, k) * rinv * ((as + a) / 2);
            wr(f->ocean_u, k, inactive ? 0.0 : txao + txio);
            wr(f->ocean_v, k, inactive ? 0.0 : tyao + tyio);
            wr(f->ocean_T, k, inactive ? 0.0 : JTao + JTio);
            wr(f->ocean_S, k, inactive ? 0.0 : Jsio);
            wr(f->ocean_eta, k, inactive ? 0.0 : Jwao + Jwio);
            wr(f->ocean_heat_content, k, inactive ? 0.0 : To * Jwao);
        }
    }
    return NESF_OK;
}

/* _assemble_net_sea_ice_fluxes! (assemble_net_sea_ice_fluxes.jl:42-81) */
int oracle_assemble_net_sea_ice_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f) {
    (void)p;
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j), kw = idx2(g, i - 1, j), ks = idx2(g, i, j - 1);
            double a = rd(f->ice_concentration, k);
            double QT = rd(f->ai_sensible, k), Qv = rd(f->ai_latent, k);
            double Qf = rdz(f->io_frazil_heat, k), Qi = rdz(f->io_interface_heat, k);
            double Js = rdz(f->snow, k);
            double SQt = (QT + Qv) * a;
            double SQb = Qf + Qi;
            int inactive = f->inactive ? f->inactive[k] != 0 : 0;
            wr(f->ice_top_heat, k, inactive ? 0.0 : SQt);
            wr(f->ice_top_snowfall, k, inactive ? 0.0 : Js);
            wr(f->ice_top_u, k, inactive ? 0.0 : (rd(f->ai_x_momentum, kw) + rd(f->ai_x_momentum, k)) / 2);
            wr(f->ice_top_v, k, inactive ? 0.0 : (rd(f->ai_y_momentum, ks) + rd(f->ai_y_momentum, k)) / 2);
            wr(f->ice_bottom_heat, k, inactive ? 0.0 : SQb);
        }
    }
    return NESF_OK;
}

/* radiation_kernels.jl:3-5 */
static inline double emitted_lw(double T, double s, double e) { double T2 = T * T; return s * e * (T2 * T2); }
static inline double absorbed_lw(double e, double L) { return -e * L; }
static inline double transmitted_sw(double a, double S) { return -(1 - a) * S; }

/* _apply_air_sea_radiative_fluxes! (apply_air_sea_radiative_fluxes.jl:62-111), no penetrating
 * shortwave forcing (shortwave_radiative_forcing returns the transmitted shortwave). */
int oracle_apply_air_sea_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    double rinv = 1 / p->ocean_reference_density, cinv = 1 / p->ocean_heat_capacity;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j);
            double a = rdz(f->ice_concentration, k);
            double Ts = rd(f->ao_interface_temperature, k) + p->interface_temperature_offset;
            double Iup = emitted_lw(Ts, p->stefan_boltzmann_constant, p->ocean_emissivity);
            double Ia = absorbed_lw(p->ocean_emissivity, rd(f->lw_down, k));
            double It = transmitted_sw(p->ocean_albedo, rd(f->sw_down, k));
            Ia *= (1 - a);
            It *= (1 - a);
            double Iup_o = Iup * (1 - a);
            double Qss = It;
            double SQ = Iup_o + Ia + Qss;
            double JT = SQ * rinv * cinv;
            int inactive = f->inactive ? f->inactive[k] != 0 : 0;
            ((double*)f->ocean_T)[k] += inactive ? 0.0 : JT;
            wr(f->ocean_upwelling_longwave, k, Iup);
            wr(f->ocean_downwelling_longwave, k, -Ia);
            wr(f->ocean_downwelling_shortwave, k, -It);
        }
    }
    return NESF_OK;
}

/* _assemble_slab_land_fluxes! (Lands/slab_land.jl:316-329): the SlabLand accumulators */
int oracle_assemble_net_land_fluxes(const nesf_land_flux_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j);
            double QT = rd(f->al_sensible, k), Qv = rd(f->al_latent, k), Jv = rd(f->al_water_vapor, k);
            double rain = rdz(f->rain, k);
            wr(f->surface_energy_flux, k, QT + Qv);
            wr(f->precipitation, k, rain + jmax(0.0, -Jv));
            wr(f->evaporation, k, jmax(0.0, Jv));
            wr(f->vapor_flux, k, Jv);
            wr(f->liquid_precipitation_flux, k, rain);
        }
    }
    return NESF_OK;
}

/* _apply_air_land_radiative_fluxes! (Radiations/apply_air_land_radiative_fluxes.jl:60-95) */
int oracle_apply_air_land_radiative_fluxes(const nesf_land_radiation_params* p, const nesf_land_flux_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j);
            double Ts = rd(f->al_interface_temperature, k);
            double Iup = emitted_lw(Ts, p->stefan_boltzmann_constant, p->land_emissivity);
            double Ia = absorbed_lw(p->land_emissivity, rd(f->lw_down, k));
            double It = transmitted_sw(p->land_albedo, rd(f->sw_down, k));
            double SQ = -Iup - (Ia + It);   /* positive into the land */
            int inactive = f->inactive ? f->inactive[k] != 0 : 0;
            ((double*)f->surface_energy_flux)[k] += inactive ? 0.0 : -SQ;
            wr(f->upwelling_longwave, k, Iup);
            wr(f->downwelling_longwave, k, -Ia);
            wr(f->downwelling_shortwave, k, -It);
        }
    }
    return NESF_OK;
}

/* _apply_air_sea_ice_radiative_fluxes! (apply_air_sea_ice_radiative_fluxes.jl:55-90) */
int oracle_apply_air_sea_ice_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f) {
    const nesf_grid* g = &f->grid;
    if (f->dtype != NESF_F64) return NESF_ERR_UNSUPPORTED;
    for (int j = 1; j <= g->ny; j++) {
        for (int i = 1; i <= g->nx; i++) {
            int64_t k = idx2(g, i, j);
            double a = rd(f->ice_concentration, k);
            double Ts = rd(f->ai_interface_temperature, k) + p->interface_temperature_offset;
            double Iup = emitted_lw(Ts, p->stefan_boltzmann_constant, p->ice_emissivity);
            double Ia = absorbed_lw(p->ice_emissivity, rd(f->lw_down, k));
            double It = transmitted_sw(p->ice_albedo, rd(f->sw_down, k));
            double SQ = (Iup + Ia + It) * a;
            int inactive = f->inactive ? f->inactive[k] != 0 : 0;
            ((double*)f->ice_top_heat)[k] += inactive ? 0.0 : SQ;
            wr(f->ice_upwelling_longwave, k, Iup);
            wr(f->ice_downwelling_longwave, k, -Ia);
            wr(f->ice_downwelling_shortwave, k, -It);
        }
    }
    return NESF_OK;
}
