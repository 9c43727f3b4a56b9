// nesf_kernels.cuh -- shared pieces of the interface-flux kernels: parameter
// conversion, array access in the Oceananigans parent layout, statistics.
#pragma once

#include <cmath>

#include "nesf_device.cuh"

namespace nesf {

// ------------------------------------------------------------ host conversion
// The stability functions' constants that the reference recomputes at every call
// (DevStab::k), in FP64.
inline void derived_stability(const nesf_stability_function& f, double* k) {
    for (int i = 0; i < 8; i++) k[i] = 0.0;
    const double* c = f.c;
    if (f.kind == NESF_PSI_EDSON_MOMENTUM || f.kind == NESF_PSI_EDSON_SCALAR) {
        const int o = f.kind == NESF_PSI_EDSON_MOMENTUM ? 5 : 6;   // A- B- C- D- E- F- from c[o]
        double Bm = c[o + 1], Em = c[o + 4];
        k[0] = 1.0 / Bm;
        k[1] = Em / 2;
        k[2] = 1.0 / Em;
        k[3] = std::sqrt(Em);
        k[4] = 1.0 / std::sqrt(Em);
    } else if (f.kind == NESF_PSI_SHEBA_PAULSON_MOMENTUM) {
        double a = c[0], b = c[1];
        double B = std::cbrt((1 - b) / b), rt3 = std::sqrt(3.0);
        k[0] = B;
        k[1] = -3 * a / b;
        k[2] = a * B / (2 * b);
        k[3] = 1.0 / (1 + B);
        k[4] = 1.0 / (1 - B + B * B);
        k[5] = 1.0 / (rt3 * B);
        k[6] = 2 * rt3;
        k[7] = std::atan((2 - B) / (rt3 * B));
    } else if (f.kind == NESF_PSI_SHEBA_PAULSON_SCALAR) {
        double a = c[0], b = c[1], cc = c[2];
        double B = std::sqrt(cc * cc - 4);
        k[0] = -b / 2;
        k[1] = b * cc / (2 * B) - a / B;
        k[2] = cc - B;
        k[3] = cc + B;
        k[4] = std::log((cc - B) / (cc + B));
    }
}

template <class R>
inline DevIface<R> make_dev_iface(const nesf_interface_params& p) {
    DevIface<R> d{};
    const nesf_thermodynamics_parameters& t = p.thermo;
    // Derived constants exactly as thermodynamic_parameters.jl:73-78,256 (double first)
    double Rd = t.gas_constant / t.dry_air_molar_mass;
    double Rv = t.gas_constant / t.water_molar_mass;
    double eps = t.dry_air_molar_mass / t.water_molar_mass;
    double cpd = Rd / t.dry_air_adiabatic_exponent;
    d.Rd = R(Rd); d.Rv = R(Rv); d.eps = R(eps); d.einv = R(1.0 / eps); d.cpd = R(cpd);
    d.cpv = R(t.water_vapor_heat_capacity); d.cpl = R(t.liquid_water_heat_capacity);
    d.cpi = R(t.water_ice_heat_capacity);
    d.Lv0 = R(t.reference_vaporization_enthalpy); d.Ls0 = R(t.reference_sublimation_enthalpy);
    d.T0 = R(t.reference_temperature); d.Ttr = R(t.triple_point_temperature); d.ptr = R(t.triple_point_pressure);
    const nesf_similarity_theory_fluxes& f = p.fluxes;
    d.vk = R(f.von_karman_constant);
    d.subgrid_kind = f.subgrid_kind;
    d.form = f.similarity_form;
    d.beta = R(f.gustiness_parameter); d.min_gust = R(f.minimum_gustiness);
    d.const_sg = R(f.constant_subgrid_velocity); d.meso_sg = R(f.mesoscale_subgrid_velocity);
    for (int n = 0; n < 3; n++) {
        d.psi[n].kind = f.stability[n].kind;
        for (int k = 0; k < 12; k++) d.psi[n].c[k] = R(f.stability[n].c[k]);
        double kd[8];
        derived_stability(f.stability[n], kd);
        for (int k = 0; k < 8; k++) d.psi[n].k[k] = R(kd[k]);
        const nesf_roughness_length& r = f.roughness[n];
        DevRough<R>& q = d.rough[n];
        q.kind = r.kind; q.wave_kind = r.wave_kind; q.visc_kind = r.viscosity_kind;
        q.value = R(r.value); q.g = R(r.gravitational_acceleration); q.nu = R(r.air_kinematic_viscosity);
        for (int k = 0; k < 4; k++) q.nuc[k] = R(r.viscosity_coefficients[k]);
        q.charnock = R(r.charnock); q.umax = R(r.wave_umax); q.c1 = R(r.wave_c1); q.c2 = R(r.wave_c2);
        q.smooth = R(r.smooth_wall_parameter); q.lmax = R(r.maximum_roughness_length);
        q.A = R(r.reynolds_A); q.b = R(r.reynolds_b);
    }
    d.d0 = R(f.zero_plane_displacement);
    d.stop_kind = f.stop_kind;
    d.maxiter = f.maxiter;
    d.tol = R(f.tolerance);
    // temperature and water vapour share a profile when their psi and roughness agree
    bool same = f.stability[1].kind == f.stability[2].kind;
    for (int k = 0; k < 12 && same; k++) same = f.stability[1].c[k] == f.stability[2].c[k];
    const nesf_roughness_length& a = f.roughness[1];
    const nesf_roughness_length& b = f.roughness[2];
    same = same && a.kind == b.kind && a.viscosity_kind == b.viscosity_kind && a.value == b.value &&
           a.air_kinematic_viscosity == b.air_kinematic_viscosity && a.reynolds_A == b.reynolds_A &&
           a.reynolds_b == b.reynolds_b && a.maximum_roughness_length == b.maximum_roughness_length;
    for (int k = 0; k < 4 && same; k++) same = a.viscosity_coefficients[k] == b.viscosity_coefficients[k];
    d.scalar_same = same ? 1 : 0;
    d.phase = p.humidity_phase;
    d.vel_form = p.velocity_formulation;
    d.temp_form = p.temperature_formulation;
    d.has_rad = p.has_radiation;
    d.x = R(p.has_water_mole_fraction ? p.water_mole_fraction : 1.0);
    d.max_dT = R(p.max_delta_T); d.k_ice = R(p.ice_conductivity); d.k_snow = R(p.snow_conductivity);
    d.kap_diff = R(p.diffusive_kappa); d.del_diff = R(p.diffusive_delta);
    d.g = R(p.gravitational_acceleration); d.h = R(p.surface_layer_height); d.hbl = R(p.boundary_layer_height);
    d.off_int = R(p.interior_temperature_offset); d.off_ifc = R(p.interface_temperature_offset);
    d.sigma = R(p.stefan_boltzmann_constant); d.alb = R(p.albedo); d.emis = R(p.emissivity);
    d.Tfw = R(p.liquidus_freshwater_melting_temperature); d.slope = R(p.liquidus_slope);
    d.rho_i = R(p.interior_reference_density); d.c_i = R(p.interior_heat_capacity);
    const bool ice = p.humidity_phase == NESF_PHASE_ICE;
    double dcp = t.water_vapor_heat_capacity - (ice ? t.water_ice_heat_capacity : t.liquid_water_heat_capacity);
    double L0 = ice ? t.reference_sublimation_enthalpy : t.reference_vaporization_enthalpy;
    d.esA = R(dcp / Rv);
    d.esK = R((L0 - dcp * t.reference_temperature) / Rv);
    d.inv_Ttr = R(1.0 / t.triple_point_temperature);
    d.hum_form = p.humidity_formulation;
    d.hum_beta = R(p.evaporation_efficiency);
    d.Sc = R(p.critical_saturation);
    d.skin_g = p.humidity_formulation == NESF_HUMIDITY_SKIN ? R(p.skin_vapor_diffusivity / p.skin_surface_thickness)
                                                            : R(0);
    d.tort = p.tortuosity;
    d.dl_max = R(p.maximum_dry_layer_depth); d.dl_Sc = R(p.dry_layer_onset_saturation);
    d.dl_eta = R(p.dry_layer_exponent); d.dl_min = R(p.minimum_dry_layer_depth);
    d.dl_D0 = R(p.molecular_diffusivity); d.dl_w = R(p.wet_transition_width); d.dl_nu = R(p.porosity);
    d.flux_form = p.flux_formulation;
    if (p.flux_formulation == NESF_FLUXES_COEFFICIENT_BASED) {
        const nesf_coefficient_fluxes& c = p.coefficients;
        d.coef_kind = c.kind;
        d.poly_mask = c.kind == NESF_COEFFICIENTS_CONSTANT ? c.polynomial_mask & 7 : 0;
        d.stop_kind = c.stop_kind;
        d.maxiter = c.maxiter;
        d.tol = R(c.tolerance);
        d.Cd = R(c.momentum); d.Ch = R(c.temperature); d.Cq = R(c.water_vapor);
        d.vk = R(c.von_karman_constant);
        d.drag_a = R(c.drag_a); d.drag_b = R(c.drag_b); d.drag_c = R(c.drag_c); d.drag_d = R(c.drag_d);
        d.U_high = R(c.high_wind_speed_threshold); d.Cd_high = R(c.high_wind_drag_coefficient);
        d.U_min = R(c.minimum_wind_speed);
        d.h0 = R(c.reference_height);
        d.Ch_stable = R(c.stable_heat_transfer_coefficient);
        d.Ch_unstable = R(c.unstable_heat_transfer_coefficient);
        d.Cq_ly = R(c.moisture_transfer_coefficient);
        // the Large-Yeager stability functions take the similarity functions' slots
        const nesf_stability_function* sf[3] = {&c.stability[0], &c.stability[1], &c.stability[1]};
        for (int n = 0; n < 3; n++) {
            d.psi[n].kind = sf[n]->kind;
            for (int k = 0; k < 12; k++) d.psi[n].c[k] = R(sf[n]->c[k]);
            double kd[8];
            derived_stability(*sf[n], kd);
            for (int k = 0; k < 8; k++) d.psi[n].k[k] = R(kd[k]);
        }
    }
    return d;
}

// ------------------------------------------------------------------ layout
struct Layout2 {
    int32_t nx, ny, hx, hy;
    int64_t sj;
    __host__ __device__ __forceinline__ int64_t at(int i, int j) const {
        return (int64_t)(i - 1 + hx) + (int64_t)(j - 1 + hy) * sj;
    }
};

template <class S> __device__ __forceinline__ double ld(const S* p, int64_t k) { return (double)__ldg(p + k); }
template <class S> __device__ __forceinline__ float ldf(const S* p, int64_t k) { return (float)__ldg(p + k); }
template <class S> __device__ __forceinline__ double ldz(const S* p, int64_t k) { return p ? (double)__ldg(p + k) : 0.0; }
template <class S, class R> __device__ __forceinline__ void st(S* p, int64_t k, R v) { if (p) p[k] = (S)v; }
// loads converted to the arithmetic type R of a kernel (the storage type of the
// streaming kernels: FP32 fields are computed in FP32, FP64 fields in FP64)
template <class R, class S> __device__ __forceinline__ R ldr(const S* p, int64_t k) { return (R)__ldg(p + k); }
template <class R, class S> __device__ __forceinline__ R ldzr(const S* p, int64_t k) { return p ? (R)__ldg(p + k) : R(0); }

// --------------------------------------------------------------- statistics
struct DevStats {
    unsigned long long cells, solved, iterations, max_iterations, nonconverged, polished, polish_iterations,
        cold_fallbacks, fp64_redo;
    unsigned long long replay_reasons[5];
    unsigned long long hist[NESF_ITER_HIST_BINS];
};

// Accumulate one cell's statistics through warp-aggregated atomics.
__device__ __forceinline__ void stats_add(DevStats* S, bool active, bool solved, int iters, bool nonconv,
                                          bool polished, int piters, bool redo, bool fallback) {
    unsigned mask = __activemask();
    unsigned a = __reduce_add_sync(mask, active ? 1u : 0u);
    unsigned s = __reduce_add_sync(mask, solved ? 1u : 0u);
    unsigned it = __reduce_add_sync(mask, solved ? (unsigned)iters : 0u);
    unsigned mx = __reduce_max_sync(mask, solved ? (unsigned)iters : 0u);
    unsigned nc = __reduce_add_sync(mask, nonconv ? 1u : 0u);
    unsigned po = __reduce_add_sync(mask, polished ? 1u : 0u);
    unsigned pi = __reduce_add_sync(mask, (unsigned)piters);
    unsigned fb = __reduce_add_sync(mask, fallback ? 1u : 0u);
    unsigned rd = __reduce_add_sync(mask, redo ? 1u : 0u);
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    if (lane == leader) {
        if (a) atomicAdd(&S->cells, (unsigned long long)a);
        if (s) atomicAdd(&S->solved, (unsigned long long)s);
        if (it) atomicAdd(&S->iterations, (unsigned long long)it);
        if (mx) atomicMax(&S->max_iterations, (unsigned long long)mx);
        if (nc) atomicAdd(&S->nonconverged, (unsigned long long)nc);
        if (po) atomicAdd(&S->polished, (unsigned long long)po);
        if (pi) atomicAdd(&S->polish_iterations, (unsigned long long)pi);
        if (fb) atomicAdd(&S->cold_fallbacks, (unsigned long long)fb);
        if (rd) atomicAdd(&S->fp64_redo, (unsigned long long)rd);
    }
    // histogram: lanes with the same bin add once through their group leader
    int bin = solved ? (iters < NESF_ITER_HIST_BINS ? iters : NESF_ITER_HIST_BINS - 1) : -1;
    unsigned grp = __match_any_sync(mask, bin);
    if (solved && lane == __ffs(grp) - 1) atomicAdd(&S->hist[bin], (unsigned long long)__popc(grp));
}

// Count a deferred replay by its reason (0..4).
__device__ __forceinline__ void stats_replay_reason(DevStats* S, int reason) {
    if (reason >= 0 && reason < 5) atomicAdd(&S->replay_reasons[reason], 1ull);
}

}  // namespace nesf
