// nesf_device.cuh -- per-cell similarity-theory physics for the interface-flux kernels.
//
// Everything here is templated on the compute type R (double for the drop-in
// FP64 solver, float for the FP32 sweep, df -- double-float, nesf_df.cuh -- for the
// adaptive solver's deferred passes). The formulas
// restate NumericalEarth.jl v0.6.2 (paths below are inside that project) and
// keep its operation order, with three kinds of exception, each moving a value
// by about an ulp (the FP64 path stays within 1e-12 of the reference): quantities
// the reference recomputes from unchanged inputs (every iteration, or every call
// of a stability function) are computed once; a division by such a quantity is a
// multiplication by its reciprocal; pow(x, y) is exp(y log x) and sums of logs
// are the log of a product. On GB300 a dependent FP64 division costs ~640
// cycles, log ~2.1k, atan ~1.9k and pow ~5.8k (an FMA 66).
#pragma once

#include <cstdint>
#include <cmath>
#include <type_traits>
#include <cuda_runtime.h>

#include "../../include/nesf.h"
#include "nesf_df.cuh"

namespace nesf {

// ------------------------------------------------------------------ math
template <class R> struct M;
template <> struct M<double> {
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
    static __device__ __forceinline__ double pow(double x, double y) { return ::pow(x, y); }
    static __device__ __forceinline__ double atan(double x) { return ::atan(x); }
    static __device__ __forceinline__ double cbrt(double x) { return ::cbrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    // Julia's min / max: NaN-propagating, -0.0 < 0.0
    static __device__ __forceinline__ double fmin(double x, double y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? x : y) : (x < y ? x : y));
    }
    static __device__ __forceinline__ double fmax(double x, double y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? y : x) : (x > y ? x : y));
    }
    static __device__ __forceinline__ double fabs(double a) { return ::fabs(a); }
    static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7ff0000000000000LL); }
    // products and sums rounded one at a time (no multiply-add contraction), as Julia rounds them
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};
template <> struct M<float> {
    static __device__ __forceinline__ float log(float x) { return ::logf(x); }
    static __device__ __forceinline__ float exp(float x) { return ::expf(x); }
    static __device__ __forceinline__ float pow(float x, float y) { return ::powf(x, y); }
    static __device__ __forceinline__ float atan(float x) { return ::atanf(x); }
    static __device__ __forceinline__ float cbrt(float x) { return ::cbrtf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
    static __device__ __forceinline__ float fmin(float x, float y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? x : y) : (x < y ? x : y));
    }
    static __device__ __forceinline__ float fmax(float x, float y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? y : x) : (x > y ? x : y));
    }
    static __device__ __forceinline__ float fabs(float a) { return ::fabsf(a); }
    static __device__ __forceinline__ float inf() { return __int_as_float(0x7f800000); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};
template <> struct M<df> {
    static __device__ __forceinline__ df log(df x) { return dfx::log(x); }
    static __device__ __forceinline__ df exp(df x) { return dfx::exp(x); }
    static __device__ __forceinline__ df pow(df x, df y) { return dfx::pow(x, y); }
    static __device__ __forceinline__ df atan(df x) { return dfx::atan(x); }
    static __device__ __forceinline__ df cbrt(df x) { return dfx::cbrt(x); }
    static __device__ __forceinline__ df sqrt(df x) { return dfx::sqrt(x); }
    static __device__ __forceinline__ df fmin(df x, df y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? x : y) : (x < y ? x : y));
    }
    static __device__ __forceinline__ df fmax(df x, df y) {
        return (isnan(x) || isnan(y)) ? x + y : (x == y ? (signbit(x) ? y : x) : (x > y ? x : y));
    }
    static __device__ __forceinline__ df fabs(df a) { return signbit(a) ? -a : a; }
    static __device__ __forceinline__ df inf() { return df(__int_as_float(0x7f800000), 0.0f); }
    static __device__ __forceinline__ df mul(df a, df b) { return a * b; }
    static __device__ __forceinline__ df add(df a, df b) { return a + b; }
};

// --------------------------------------------------------- device parameters
// c: the coefficients (nesf_stability_function); k: constants derived from them on
// the host, which the reference recomputes at every call (make_dev_iface):
//   Edson (both):  1/B-, E-/2, 1/E-, sqrt(E-), 1/sqrt(E-)
//   SHEBA momentum: B = cbrt((1-b)/b), -3a/b, aB/(2b), 1/(1+B), 1/(1-B+B^2),
//                   1/(sqrt3 B), 2 sqrt3, atan((2-B)/(sqrt3 B))
//   SHEBA scalar:  -b/2, bc/(2B) - a/B, c-B, c+B, log((c-B)/(c+B)) with B = sqrt(c^2-4)
template <class R> struct DevStab {
    int32_t kind;
    R c[12];
    R k[8];
};

template <class R> struct DevRough {
    int32_t kind, wave_kind, visc_kind;
    R value, g, nu, nuc[4], charnock, umax, c1, c2, smooth, lmax, A, b;
};

// Flattened nesf_interface_params with the derived thermodynamic constants
// (thermodynamic_parameters.jl:73-78, 256) evaluated once on the host.
template <class R> struct DevIface {
    // thermodynamics
    R Rd, Rv, eps, einv, cpd, cpv, cpl, cpi, Lv0, Ls0, T0, Ttr, ptr;
    // similarity theory
    R vk;
    int32_t subgrid_kind, form;
    R beta, min_gust, const_sg, meso_sg;
    DevStab<R> psi[3];
    DevRough<R> rough[3];
    R d0;
    int32_t stop_kind, maxiter;
    R tol;
    int32_t scalar_same;      // temperature and vapour share roughness and psi
    // interface properties
    int32_t phase, vel_form, temp_form, has_rad;
    R x;                      // water mole fraction (1 when `nothing`)
    R max_dT, k_ice, k_snow, kap_diff, del_diff;
    R g, h, hbl, off_int, off_ifc;
    R sigma, alb, emis, Tfw, slope, rho_i, c_i;
    // ln e_sat(T) = ln p_tr + esA ln(T / T_tr) + esK (1 / T_tr - 1 / T) for the interface's
    // phase: esA = (cp_v - cp_c) / R_v, esK = (L_0 - (cp_v - cp_c) T_0) / R_v; inv_Ttr = 1 / T_tr
    R esA, esK, inv_Ttr;
    // CoefficientBasedFluxes (flux_form 1): its stop criteria are in stop_kind / maxiter / tol,
    // Large-Yeager's von Karman constant in vk and its stability functions in psi[0] (momentum)
    // and psi[1], psi[2] (scalar)
    int32_t flux_form, coef_kind, poly_mask;
    R Cd, Ch, Cq;                         // constant transfer coefficients
    R drag_a, drag_b, drag_c, drag_d;     // PolynomialNeutralDragCoefficient
    R U_high, Cd_high, U_min;
    R h0, Ch_stable, Ch_unstable, Cq_ly;  // reference height, Stanton/Dalton factors
    // land surface humidity (nesf_humidity_formulation): constant efficiency, critical
    // saturation (> 0: CriticalSaturation), soil vapor conductance kappa_q / d; DryLayerHumidity:
    // tortuosity model, maximum depth, onset saturation, exponent, minimum depth, D_0, blend
    // width, porosity
    int32_t hum_form, tort;
    R hum_beta, Sc, skin_g;
    R dl_max, dl_Sc, dl_eta, dl_min, dl_D0, dl_w, dl_nu;
};

// ------------------------------------------------------------- thermodynamics
// Thermodynamics.jl restatements (saturation_vapor_pressure, air_density, cp_m,
// latent heats, virtual temperature) with the parameter set of
// src/Atmospheres/thermodynamic_parameters.jl.

// saturation_vapor_pressure, e_sat = p_tr (T / T_tr)^A exp(K (1 / T_tr - 1 / T))
// (docs/src/interface_fluxes.md:86-97, A = (cp_v - cp_c) / R_v, K = (L_0 - (cp_v -
// cp_c) T_0) / R_v for the interface's phase). The FP64 iterations keep this
// two-factor form: q_a - q_s(T_s) can cancel, and the difference multiplies the
// rounding of e_sat by q_s / (q_a - q_s).
template <class R>
__device__ __forceinline__ R esat(const DevIface<R>& P, R T) {
    return P.ptr * M<R>::pow(T / P.Ttr, P.esA) * M<R>::exp(P.esK * (R(1) / P.Ttr - R(1) / T));
}

// The same as one exponential, p_tr exp(A ln(T / T_tr) + K (T - T_tr) / (T_tr T)):
// a log and an exp in place of pow and exp (FP64 pow costs ~5.8k cycles per
// dependent call on this GPU, log + exp ~3k), within a few ulps of esat. The FP32
// solvers' FP64 anchors use it (their own rounding is ~1e-7).
template <class R>
__device__ __forceinline__ R esat_exp(const DevIface<R>& P, R T) {
    return P.ptr * M<R>::exp(P.esA * M<R>::log(T * P.inv_Ttr) + P.esK * ((T - P.Ttr) * P.inv_Ttr) / T);
}

template <class R> __device__ __forceinline__ R gas_constant_air(const DevIface<R>& P, R q) {
    return P.Rd * (R(1) + (P.eps - R(1)) * q);
}
template <class R> __device__ __forceinline__ R air_density(const DevIface<R>& P, R T, R p, R q) {
    return p / (gas_constant_air(P, q) * T);
}
template <class R> __device__ __forceinline__ R cp_m(const DevIface<R>& P, R q) {
    return P.cpd + (P.cpv - P.cpd) * q;
}
template <class R> __device__ __forceinline__ R latent_heat_vapor(const DevIface<R>& P, R T) {
    return P.Lv0 + (P.cpv - P.cpl) * (T - P.T0);
}
template <class R> __device__ __forceinline__ R latent_heat_sublim(const DevIface<R>& P, R T) {
    return P.Ls0 + (P.cpv - P.cpi) * (T - P.T0);
}
template <class R> __device__ __forceinline__ R virtual_temperature(const DevIface<R>& P, R T, R q) {
    return gas_constant_air(P, q) / P.Rd * T;
}

// surface_specific_humidity(::ImpureSaturationSpecificHumidity)
// (InterfaceComputations/interface_states.jl:55-74); EXP: e_sat from esat_exp, which FP32
// (classification, network features) and double-float (the replays) always take.
template <class R, bool EXP = false>
__device__ __forceinline__ R surface_specific_humidity(const DevIface<R>& P, R pa, R Ts) {
    R pv = P.x * ((EXP || !std::is_same<R, double>::value) ? esat_exp(P, Ts) : esat(P, Ts));
    pv = M<R>::fmin(pv, R(0.999) * pa);
    return P.einv * pv / (pa - (R(1) - P.einv) * pv);
}

// Land surface humidity at a fixed T_s (compute_interface_humidity, interface_states.jl:587-598):
// BulkHumidity q_sat where the saturation S > 0, else 0 (:120-125); FractionalHumidity
// beta q_sat with beta a constant or min(S / S_c, 1) (CriticalSaturation, :152-158).
// q_sat is the pressure-based saturation humidity (:76-90): x = 1 for land.
template <class R>
__device__ __forceinline__ R land_humidity(const DevIface<R>& P, R pa, R Ts, R S) {
    R qsat = surface_specific_humidity(P, pa, Ts);
    if (P.hum_form == NESF_HUMIDITY_BULK) return S > R(0) ? qsat : R(0);
    R beta = P.Sc > R(0) ? M<R>::fmin(S / P.Sc, R(1)) : P.hum_beta;
    return beta * qsat;
}

// The land surface humidity iterated with the fluxes, from the previous iterate: a vapor
// flux G (q_src - q_s) from a source at q_src balances the atmospheric flux J = -rho u* q*,
// written with dq = q_s_prev - q_a so that it stays finite as dq -> 0. SkinHumidity
// (interface_states.jl:626-651): G = kappa_q / d, q_src the reservoir's saturation.
// DryLayerHumidity (dry_layer_humidity.jl:339-365): G = rho D_eff / max(delta, delta_min), q_src
// the front's saturation, and the series solution is blended with the saturated skin q_wet by
// the logistic weight sig; with the interface at the bulk land temperature q_src = q_wet.
// The sums cancel where q_s is close to q_a; each product and sum is rounded on its own, as
// the reference rounds them, so the FP64 path stays on the reference's iterates.
template <class R>
__device__ __forceinline__ R balance_humidity(const DevIface<R>& P, R rho, R qa, R qsrc, R G, R sig, R qs_prev,
                                              R us, R qst) {
    using Mr = M<R>;
    R Ja = -Mr::mul(Mr::mul(rho, us), qst);
    R dq = qs_prev - qa;
    R D = Mr::add(Mr::mul(G, dq), Ja);
    R qs = Mr::add(Mr::mul(Mr::mul(G, qsrc), dq), Mr::mul(Ja, qa)) / D;
    qs = D == R(0) ? qs_prev : qs;
    if (P.hum_form == NESF_HUMIDITY_DRY_LAYER) qs = Mr::add(qsrc, Mr::mul(sig, qs - qsrc));
    return qs;
}

// surface_atmosphere_temperature (interface_states.jl:308-317)
template <class R>
__device__ __forceinline__ R surface_atmosphere_temperature(const DevIface<R>& P, R Ta, R qa) {
    R c = cp_m(P, qa);
    return Ta + P.g * P.h / c;
}

// -------------------------------------------------------- stability functions
// similarity_theory_turbulent_fluxes.jl. The reference evaluates both branches
// and selects with ifelse(zeta < 0, ...); here only the selected branch is
// evaluated, which gives the same value. Division by a coefficient is
// multiplication by its host-derived reciprocal, sums of logarithms are the
// logarithm of a product, and pow is exp(y log x): each moves a result by about an
// ulp, and the FP64 division, log, atan and pow they save cost 0.6k-5.8k cycles per
// dependent call.

// Convective branch (zeta < 0) of Edson's momentum (MOM) and scalar functions
// (:501-532, :586-618): (1 - f) psi1 + f psi2, f = zeta^2 / (1 + zeta^2).
template <class R, bool MOM>
__device__ __forceinline__ R edson_unstable(R Am, R Bm, R iBm, R Cm, R Dm, R hEm, R iEm, R sE, R isE, R Fm, R z) {
    R zm = M<R>::fmin(R(0), z);
    R psi1;
    if (MOM) {
        R f1 = M<R>::sqrt(M<R>::sqrt(R(1) - Am * zm));
        psi1 = Bm * M<R>::log((R(1) + f1) * iBm) + M<R>::log((R(1) + f1 * f1) * iBm) - Bm * M<R>::atan(f1) + Cm;
    } else {
        R f1 = M<R>::sqrt(R(1) - Am * zm);
        psi1 = Bm * M<R>::log((R(1) + f1) * iBm) + Cm;
    }
    R f2 = M<R>::cbrt(R(1) - Dm * zm);
    R psi2 = hEm * M<R>::log((R(1) + f2 + f2 * f2) * iEm) - sE * M<R>::atan((R(1) + R(2) * f2) * isE) + Fm;
    R f = zm * zm / (R(1) + zm * zm);
    return (R(1) - f) * psi1 + f * psi2;
}

// Stable branch (zeta >= 0) of Edson's momentum (MOM) and scalar functions.
template <class R, bool MOM>
__device__ __forceinline__ R edson_stable(const DevStab<R>& s, R z) {
    const R* c = s.c;
    R zmax = c[0], Ap = c[1], Bp = c[2], Cp = c[3], Dp = c[4];
    R zp = M<R>::fmax(R(0), z);
    R dz = M<R>::fmin(zmax, Ap * zp);
    if (MOM) return -Bp * zp - Cp * (zp - Dp) * M<R>::exp(-dz) - Cp * Dp;
    R x = R(1) + Bp * zp;
    R xC = Cp == R(1.5) ? x * M<R>::sqrt(x) : M<R>::exp(Cp * M<R>::log(x));   // x^Cp
    return -xC - Bp * (zp - Dp) * M<R>::exp(-dz) - c[5];
}

template <class R>
__device__ __forceinline__ R sheba_momentum(const R* k, R z) {     // :643-657
    R zp = M<R>::fmax(R(0), z);
    R x = M<R>::cbrt(R(1) + zp);
    R B = k[0];
    R P1 = k[1] * (x - R(1));
    R u = (x + B) * k[3], v = (x * x - B * x + B * B) * k[4];
    R P2 = k[2] * (M<R>::log(u * u / v) + k[6] * (M<R>::atan((R(2) * x - B) * k[5]) - k[7]));
    return P1 + P2;
}

template <class R>
__device__ __forceinline__ R sheba_scalar(R c, const R* k, R z) {  // :665-677
    R zp = M<R>::fmax(R(0), z);
    R P1 = k[0] * M<R>::log(R(1) + c * zp + zp * zp);
    R P2 = k[1] * (M<R>::log((R(2) * zp + k[2]) / (R(2) * zp + k[3])) - k[4]);
    return P1 + P2;
}

template <class R>
__device__ __forceinline__ R paulson_momentum(R a, R b, R z) {   // :688-699
    R zm = M<R>::fmin(R(0), z);
    R x = M<R>::sqrt(M<R>::sqrt(R(1) - a * zm));
    R u = (R(1) + x) * R(0.5);
    R P12 = M<R>::log(u * u * ((R(1) + x * x) * R(0.5)));   // 2 log(u) + log((1 + x^2) / 2)
    R P3 = -R(2) * M<R>::atan(x);
    return P12 + P3 + b;
}

template <class R>
__device__ __forceinline__ R paulson_scalar(R a, R z) {          // :705-710
    R zm = M<R>::fmin(R(0), z);
    R x = M<R>::sqrt(M<R>::sqrt(R(1) - a * zm));
    return R(2) * M<R>::log((R(1) + x * x) * R(0.5));
}

template <class R>
__device__ __forceinline__ R psi_linear(R coef, R zmax, R z) {       // :747-752
    R zp = M<R>::fmax(R(0), z);
    return -coef * M<R>::fmin(zp, zmax);
}

// One out-of-line copy of each function per kernel (the solves' loops call them from
// several places; inlined, the kernels outgrow the instruction cache).
template <class R, bool MOM>
__device__ __noinline__ R psi_edson_unstable(R Am, R Bm, R iBm, R Cm, R Dm, R hEm, R iEm, R sE, R isE, R Fm, R z) {
    return edson_unstable<R, MOM>(Am, Bm, iBm, Cm, Dm, hEm, iEm, sE, isE, Fm, z);
}

template <class R>
__device__ __noinline__ R psi_sheba_momentum(R k0, R k1, R k2, R k3, R k4, R k5, R k6, R k7, R z) {
    const R k[8] = {k0, k1, k2, k3, k4, k5, k6, k7};
    return sheba_momentum(k, z);
}

template <class R>
__device__ __noinline__ R psi_sheba_scalar(R c, R k0, R k1, R k2, R k3, R k4, R z) {
    const R k[5] = {k0, k1, k2, k3, k4};
    return sheba_scalar(c, k, z);
}

template <class R>
__device__ __noinline__ R psi_paulson_momentum(R a, R b, R z) { return paulson_momentum(a, b, z); }

template <class R>
__device__ __noinline__ R psi_paulson_scalar(R a, R z) { return paulson_scalar(a, z); }

// stability_profile dispatch; SplitStabilityFunction (:720-725) takes the stable
// branch for z > 0, Edson's functions select with z < 0.
template <class R>
__device__ __forceinline__ R stability(const DevStab<R>& s, R z) {
    const R* c = s.c;
    const R* k = s.k;
    switch (s.kind) {
    case NESF_PSI_EDSON_MOMENTUM:
        if (z < R(0)) return psi_edson_unstable<R, true>(c[5], c[6], k[0], c[7], c[8], k[1], k[2], k[3], k[4], c[10], z);
        return edson_stable<R, true>(s, z);
    case NESF_PSI_EDSON_SCALAR:
        if (z < R(0))
            return psi_edson_unstable<R, false>(c[6], c[7], k[0], c[8], c[9], k[1], k[2], k[3], k[4], c[11], z);
        return edson_stable<R, false>(s, z);
    case NESF_PSI_SHEBA_PAULSON_MOMENTUM:
        return z > R(0) ? psi_sheba_momentum(k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], z)
                        : psi_paulson_momentum(c[2], c[3], z);
    case NESF_PSI_SHEBA_PAULSON_SCALAR:
        return z > R(0) ? psi_sheba_scalar(c[2], k[0], k[1], k[2], k[3], k[4], z) : psi_paulson_scalar(c[3], z);
    case NESF_PSI_LINEAR_PAULSON_MOMENTUM:
        return z > R(0) ? psi_linear(c[0], c[1], z) : psi_paulson_momentum(c[2], c[3], z);
    case NESF_PSI_LINEAR_PAULSON_SCALAR:
        return z > R(0) ? psi_linear(c[0], c[1], z) : psi_paulson_scalar(c[2], z);
    default: return R(0);
    }
}

// similarity_profile (:242-253), with 1 / L in place of L (h / L = h * (1 / L)); the
// COARE form has no psi(l / L) term.
template <class R>
__device__ __forceinline__ R similarity_profile(int form, const DevStab<R>& psi, R h, R l, R invL) {
    R zeta = h * invL;
    R ph = stability(psi, zeta);
    if (form == NESF_PROFILE_COARE) return M<R>::log(h / l) - ph;
    R pl = stability(psi, l * invL);
    return M<R>::log(h / l) - ph + pl;
}

// ---------------------------------------------------------- roughness lengths
// roughness_lengths.jl:182-189 (viscosity), 197-210 (momentum), 231-246 (scalar)
template <class R>
__device__ __forceinline__ R air_viscosity(const DevRough<R>& r, R T) {
    if (r.visc_kind == 0) return r.nu;
    R Tc = T - R(273.15);
    return r.nuc[0] + r.nuc[1] * Tc + r.nuc[2] * Tc * Tc + r.nuc[3] * (Tc * Tc * Tc);
}

template <class R>
__device__ __forceinline__ R momentum_roughness(const DevRough<R>& r, R us, R U, R nu) {
    if (r.kind == NESF_ROUGHNESS_CONSTANT) return r.value;
    R Cg = r.charnock;
    if (r.wave_kind == 1) Cg = M<R>::fmax(R(0), r.c1 * M<R>::fmin(U, r.umax) + r.c2);
    R lW = Cg * (us * us) / r.g;
    R lR = r.smooth == R(0) ? R(0) : r.smooth * nu / us;
    return M<R>::fmin(lW + lR, r.lmax);
}

template <class R>
__device__ __forceinline__ R scalar_roughness(const DevRough<R>& r, R lu, R us, R nu) {
    if (r.kind == NESF_ROUGHNESS_CONSTANT) return r.value;
    R Rs = lu * us / nu;
    R ls = Rs == R(0) ? R(0) : r.A * M<R>::exp(-r.b * M<R>::log(Rs));   // A / Rs^b
    return M<R>::fmin(ls, r.lmax);
}

// vsgs2 (similarity_theory_turbulent_fluxes.jl:88-98)
template <class R>
__device__ __forceinline__ R vsgs2(const DevIface<R>& P, R us, R bs) {
    R conv = R(0);
    if (P.subgrid_kind == NESF_SUBGRID_CONSTANT) {
        conv = P.const_sg * P.const_sg;
    } else if (P.subgrid_kind == NESF_SUBGRID_CONVECTIVE) {
        R Jb = -us * bs;
        // a stable or neutral cell has no buoyancy flux to take the cube root of: cbrt(0) = 0
        // exactly, and the cube root is the iteration's dearest call after pow in FP64
        R wb = M<R>::fmax(R(0), Jb) * P.hbl;
        R UG = M<R>::fmax(P.min_gust, P.beta * (wb != R(0) ? M<R>::cbrt(wb) : wb));
        conv = UG * UG;
    }
    return conv + P.meso_sg * P.meso_sg;
}

// ------------------------------------------------------------ the fixed point
// Per-cell state the iteration needs and that does not change between
// iterations (for BulkTemperature everything that depends on T_s).
template <class R> struct CellConst {
    R ua, va, Ta, pa, qa;        // atmosphere
    R ui, vi;                    // interface velocities
    R Ti, Si;                    // interior temperature (K) and salinity
    R hi, hs, hc;                // ice state (conductive skin)
    R sw, lw, kappa;             // radiation, interior diffusivity (<0: none)
    R du, dv, dU2;               // velocity difference and its square norm
    R tha;                       // surface_atmosphere_temperature
    R rho_a, cp_a, L_s;          // air density, cp_m, latent_heat_sublim (skin only)
    R Rth;                       // conductive resistance h_s / k_s + h_i / k_i (ice skin only)
    R qres;                      // land q_sat at the bulk land temperature (SKIN, DRY_LAYER source)
    R Gq, sig;                   // SKIN, DRY_LAYER: vapor conductance; DRY_LAYER: blend weight
};

// The ice and snow layers' thermal resistance (interface_states.jl:468-524), fixed
// over the iteration.
template <class R>
__device__ __forceinline__ R conductive_resistance(const DevIface<R>& P, R hs, R hi) {
    return P.k_snow > R(0) ? hs / P.k_snow + hi / P.k_ice : hi / P.k_ice;
}

// Quantities that depend on the interface temperature.
template <class R> struct SurfaceConst {
    R Ts, qs, dth, dq;
    R gTv, A1, A2;   // b* = gTv * (theta* A1 + A2 q*)   (buoyancy_scale, :417-425)
    R nu_u, nu_t, nu_q;
};

template <class R>
__device__ __forceinline__ void surface_const(const DevIface<R>& P, const CellConst<R>& c, R Ts, R qs,
                                              SurfaceConst<R>& s) {
    s.Ts = Ts;
    s.qs = qs;
    s.dq = c.qa - qs;
    s.dth = c.tha - Ts;
    R Tv = virtual_temperature(P, Ts, qs);
    R delta = P.eps - R(1);
    s.gTv = P.g / Tv;
    s.A1 = R(1) + delta * qs;
    s.A2 = delta * Tv;
    s.nu_u = air_viscosity(P.rough[0], Ts);
    s.nu_t = air_viscosity(P.rough[1], Ts);
    s.nu_q = air_viscosity(P.rough[2], Ts);
}

// PolynomialNeutralDragCoefficient (coefficient_based_turbulent_fluxes.jl:48-54), U^6 as (U^3)^2.
template <class R>
__device__ __forceinline__ R neutral_drag(const DevIface<R>& P, R U) {
    U = M<R>::fmax(U, P.U_min);
    R U3 = U * U * U;
    return U < P.U_high ? (P.drag_a / U + P.drag_b + P.drag_c * U - P.drag_d * (U3 * U3)) / R(1000) : P.Cd_high;
}

// iterate_interface_fluxes(::CoefficientBasedFluxes) (coefficient_based_turbulent_fluxes.jl:346-371)
// with evaluate_coefficients for constants (:269-285) or Large-Yeager (:288-340). Delta h is
// the surface layer height (compute_interface_state.jl:101). Inlined: P is a kernel parameter,
// whose address an out-of-line call would copy to local memory.
template <class R>
__device__ __forceinline__ void coefficient_fluxes(const DevIface<R>& P, R dU2, R gTv, R A1, R A2, R dth, R dq, R us,
                                                R ts, R qst, R& us_n, R& ts_n, R& qs_n) {
    const bool ly = P.coef_kind == NESF_COEFFICIENTS_LARGE_YEAGER;
    R dU = M<R>::fmax(M<R>::sqrt(dU2), ly ? P.U_min : R(0));
    R Cd = P.Cd, Ch = P.Ch, Cq = P.Cq;
    if (P.poly_mask) {   // PolynomialNeutralDragCoefficient slots of a constant SimilarityScales (:271)
        R Cp = neutral_drag(P, dU);
        if (P.poly_mask & 1) Cd = Cp;
        if (P.poly_mask & 2) Ch = Cp;
        if (P.poly_mask & 4) Cq = Cp;
    }
    if (ly) {
        const R k = P.vk, dh = P.h;
        R bs = gTv * (ts * A1 + A2 * qst);                 // buoyancy_scale (:308)
        R zeta = bs == R(0) ? R(0) : dh * (k * bs) / (us * us);   // dh / L, L = u*^2 / (k b*)
        R psim = stability(P.psi[0], zeta);
        R psih = stability(P.psi[1], zeta);
        R lg = M<R>::log(dh / P.h0);
        R Cdp = us == R(0) ? neutral_drag(P, dU) : us * us / (dU * dU);
        R UN10 = dU / (R(1) + M<R>::sqrt(Cdp) / k * (lg - psim));
        UN10 = M<R>::fmax(UN10, P.U_min);
        R CdN = neutral_drag(P, UN10);
        R sCdN = M<R>::sqrt(CdN);
        R ChN = sCdN / R(1000) * (zeta > R(0) ? P.Ch_stable : P.Ch_unstable);
        R CqN = sCdN / R(1000) * P.Cq_ly;
        R xim = sCdN / k * (lg - psim);
        Cd = CdN / ((R(1) + xim) * (R(1) + xim));
        R xih = sCdN / k * (lg - psih);
        R ratio = M<R>::sqrt(Cd) / sCdN;
        Ch = ChN * ratio / (R(1) + ChN * xih);
        Cq = CqN * ratio / (R(1) + CqN * xih);
    }
    R sCd = M<R>::sqrt(Cd);
    us_n = sCd * dU;
    ts_n = Cd == R(0) ? R(0) : Ch / sCd * dth;
    qs_n = Cd == R(0) ? R(0) : Cq / sCd * dq;
}

// Two lanes of a warp on one cell (the FP64 replays): `half` 0 or 1, `mask` the pair's lanes.
struct LanePair {
    unsigned mask;
    int half;
};

// iterate_interface_fluxes(::SimilarityTheoryFluxes) (:315-385), or the coefficient-based
// formulation's when the interface uses it. PAIR: the two lanes of `lp` iterate the same
// cell and split the logarithmic profiles' four stability-function values and two
// logarithms between them -- lane 0 psi(h / L) and log(h / l_u), lane 1 psi(l / L) and
// log(h / l_t) -- each by the same function and expression as the single-lane path, then
// exchange them: a dependent FP64 chain (one cell's iterations, ~64 cycles per dependent
// FP64 instruction) shortens by the split part.
template <class R, bool PAIR = false>
__device__ __forceinline__ void iterate_fluxes(const DevIface<R>& P, const CellConst<R>& c, const SurfaceConst<R>& s,
                                               R us, R ts, R qst, R& us_n, R& ts_n, R& qs_n,
                                               LanePair lp = LanePair{0u, 0}) {
    if (__builtin_expect(P.flux_form == NESF_FLUXES_COEFFICIENT_BASED, 0)) {   // off the hot path's layout
        coefficient_fluxes(P, c.dU2, s.gTv, s.A1, s.A2, s.dth, s.dq, us, ts, qst, us_n, ts_n, qs_n);
        return;
    }
    R bs = s.gTv * (ts * s.A1 + s.A2 * qst);
    R Usg2 = vsgs2(P, us, bs);
    R U = M<R>::sqrt(c.dU2 + Usg2);
    R lu = momentum_roughness(P.rough[0], us, U, s.nu_u);
    R lt = scalar_roughness(P.rough[1], lu, us, s.nu_t);
    R h = M<R>::fmax(P.h - P.d0, R(2) * lu);
    // 1 / L, L = u*^2 / (kappa b*) (Inf when b* = 0)
    R invL = bs == R(0) ? R(0) : (P.vk * bs) / (us * us);
    R chiu, chit;
    if (PAIR && P.form != NESF_PROFILE_COARE) {
        const bool hi = lp.half != 0;
        const R pm = stability(P.psi[0], (hi ? lu : h) * invL);
        const R ph = stability(P.psi[1], (hi ? lt : h) * invL);
        const R lg = M<R>::log(h / (hi ? lt : lu));
        const R pm2 = __shfl_xor_sync(lp.mask, pm, 1);
        const R ph2 = __shfl_xor_sync(lp.mask, ph, 1);
        const R lg2 = __shfl_xor_sync(lp.mask, lg, 1);
        // similarity_profile's log(h / l) - psi(h / L) + psi(l / L), in its order
        chiu = P.vk / ((hi ? lg2 : lg) - (hi ? pm2 : pm) + (hi ? pm : pm2));
        chit = P.vk / ((hi ? lg : lg2) - (hi ? ph2 : ph) + (hi ? ph : ph2));
    } else {
        chiu = P.vk / similarity_profile(P.form, P.psi[0], h, lu, invL);
        chit = P.vk / similarity_profile(P.form, P.psi[1], h, lt, invL);
    }
    R chiq;
    if (P.scalar_same) {
        chiq = chit;
    } else {
        R lq = scalar_roughness(P.rough[2], lu, us, s.nu_q);
        chiq = P.vk / similarity_profile(P.form, P.psi[2], h, lq, invL);
    }
    us_n = chiu * U;
    ts_n = chit * s.dth;
    qs_n = chiq * s.dq;
}

// Julia clamp: ifelse(x > hi, hi, ifelse(x < lo, lo, x))
template <class R> __device__ __forceinline__ R clampr(R x, R lo, R hi) {
    return x > hi ? hi : (x < lo ? lo : x);
}

// compute_interface_temperature(::SkinTemperature) (interface_states.jl:526-577) with
// flux_balance_temperature (434-457 diffusive, 468-524 conductive ice/snow).
// `pinned` is set when the result is fixed by the melting-point cap or the
// unconsolidated-ice branch (T_s does not depend on the fluxes there).
template <class R>
__device__ __forceinline__ R skin_temperature(const DevIface<R>& P, const CellConst<R>& c, R Tm1, R us, R ts, R qst,
                                              bool* pinned = nullptr) {
    R sigma = P.has_rad ? P.sigma : R(0);
    R eps = P.has_rad ? P.emis : R(0);
    R alb = P.has_rad ? P.alb : R(0);
    R SW = P.has_rad ? c.sw : R(0);
    R LW = P.has_rad ? c.lw : R(0);
    R T2 = Tm1 * Tm1;
    R Iup = sigma * eps * (T2 * T2);
    R Qd = -(R(1) - alb) * SW - eps * LW;
    R QT = -c.rho_a * c.cp_a * us * ts;
    R Qv = -c.rho_a * c.L_s * us * qst;
    R Tat = c.tha;
    if (P.temp_form == NESF_SKIN_TEMPERATURE_DIFFUSIVE) {
        R kap = c.kappa >= R(0) ? M<R>::fmax(c.kappa, P.kap_diff) : P.kap_diff;
        R del = P.del_diff;
        R Qa = Qv + Iup + Qd;
        R lam = R(1) / (P.rho_i * P.c_i);
        R JT = Qa * lam;
        R dT = Tat - Tm1;
        R OmT = QT * lam;
        R D = kap * dT - OmT * del;
        R Tst = (c.Ti * kap * dT - (JT * dT + OmT * Tat) * del) / D;
        Tst = D == R(0) ? Tm1 : Tst;
        return c.Ti + clampr(Tst - c.Ti, -P.max_dT, P.max_dT);
    }
    R Rth = c.Rth;
    R Tb = P.Tfw - P.slope * c.Si;
    Tb = Tb + P.off_ifc;
    R dT = Tat - Tm1;
    R Qa = Qv + Iup + Qd;
    R Om = dT == R(0) ? R(0) : QT / dT;
    R beta = R(4) * Iup / Tm1;
    R D = R(1) + beta * Rth - Om * Rth;
    R Tst = (Tb + beta * Rth * Tm1 - Om * Rth * Tat - Qa * Rth) / D;
    Tst = D == R(0) ? Tm1 : Tst;
    Tst = isnan(Tst) ? Tm1 : Tst;
    R Tp = Tm1 + clampr(Tst - Tm1, -P.max_dT, P.max_dT);
    R Tm = P.Tfw + P.off_ifc;
    if (pinned) *pinned = !(Tp < Tm) || !(c.hi >= c.hc);
    Tp = M<R>::fmin(Tp, Tm);
    return c.hi >= c.hc ? Tp : Tb;
}

// One iterate_interface_state (compute_interface_state.jl:69-122). For the bulk
// formulation `s` is fixed; for skin formulations it is rebuilt from the new T_s.
// QSKIN (land SkinHumidity, DryLayerHumidity): T_s fixed, q_s iterated from the previous iterate; a template
// flag so that the other solves carry none of its code or registers.
template <class R, bool SKIN, bool QSKIN = false, bool PAIR = false>
__device__ __forceinline__ void iterate_state(const DevIface<R>& P, const CellConst<R>& c, SurfaceConst<R>& s,
                                              R& us, R& ts, R& qst, bool* pinned = nullptr,
                                              LanePair lp = LanePair{0u, 0}) {
    if (SKIN) {
        R Ts = skin_temperature(P, c, s.Ts, us, ts, qst, pinned);
        R qs = surface_specific_humidity(P, c.pa, Ts);
        surface_const(P, c, Ts, qs, s);
    } else if (QSKIN) {   // T_s fixed, q_s iterated
        R qs = balance_humidity(P, c.rho_a, c.qa, c.qres, c.Gq, c.sig, s.qs, us, qst);
        surface_const(P, c, s.Ts, qs, s);
    }
    R a, b, d;
    iterate_fluxes<R, PAIR>(P, c, s, us, ts, qst, a, b, d, lp);
    us = a;
    ts = b;
    qst = d;
}

// compute_interface_state with ConvergenceStopCriteria / FixedIterations
// (compute_interface_state.jl:10-24, 31-58). Returns the iteration count; the
// last drift is left in `drift`.
template <class R, bool SKIN, bool QSKIN = false, bool PAIR = false>
__device__ __forceinline__ int fixed_point(const DevIface<R>& P, const CellConst<R>& c, SurfaceConst<R>& s,
                                           R& us, R& ts, R& qst, int maxiter, R& drift,
                                           LanePair lp = LanePair{0u, 0}) {
    int it = 0;
    drift = M<R>::inf();
    if (P.stop_kind == NESF_STOP_FIXED_ITERATIONS) {
        for (; it < maxiter; it++) iterate_state<R, SKIN, QSKIN, PAIR>(P, c, s, us, ts, qst, nullptr, lp);
        return it;
    }
    do {
        R u0 = us, t0 = ts, q0 = qst;
        iterate_state<R, SKIN, QSKIN, PAIR>(P, c, s, us, ts, qst, nullptr, lp);
        it++;
        drift = M<R>::fabs(us - u0) + M<R>::fabs(ts - t0) + M<R>::fabs(qst - q0);
    } while (!(drift < P.tol) && it < maxiter);
    return it;
}

}  // namespace nesf
