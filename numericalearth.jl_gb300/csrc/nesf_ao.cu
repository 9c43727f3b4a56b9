// nesf_ao.cu -- atmosphere-ocean similarity-theory solve.
//
// _compute_atmosphere_ocean_interface_state! (InterfaceComputations/atmosphere_ocean_fluxes.jl:80-197)
//
// One thread per surface cell over the halo ring (0:nx+1, 0:ny+1), SoA loads of
// the Oceananigans parent arrays (i fastest, so a warp reads 32 consecutive
// cells of a row). Pass 0 writes the land cells and compacts the others into a
// work list split by stability class; pass 1 solves the listed cells (PLAIN:
// FP64; POLISH: FP32 sweep + FP64 Newton); pass 2 replays, packed into full
// warps, the POLISH cells that must follow the reference's FP64 iteration.
#include "nesf_solve.cuh"

namespace nesf {

// assemble_interior_state + the atmosphere reads (atmosphere_ocean_fluxes.jl:62-71, 97-128)
// R: double (the reference's FP64 iteration) or df (the adaptive solver's replays).
template <class S, class R>
__device__ __forceinline__ void ao_load(const DevIface<R>& P, const AOArgs<S>& a, int64_t k, bool skin,
                                        CellConst<R>& c, bool& land) {
    c.ua = ldr<R>(a.ua, k); c.va = ldr<R>(a.va, k); c.Ta = ldr<R>(a.Ta, k); c.pa = ldr<R>(a.pa, k);
    c.qa = ldr<R>(a.qa, k);
    c.ui = (ldr<R>(a.uo, k) + ldr<R>(a.uo, k + 1)) / R(2);         // centre average of the x-face velocity
    c.vi = (ldr<R>(a.vo, k) + ldr<R>(a.vo, k + a.L.sj)) / R(2);    // centre average of the y-face velocity
    c.Ti = ldr<R>(a.To, k) + P.off_int;
    c.Si = ldr<R>(a.So, k);
    c.hi = c.hs = c.hc = R(0);
    c.Rth = R(0);
    c.sw = ldzr<R>(a.sw, k);
    c.lw = ldzr<R>(a.lw, k);
    c.kappa = a.kappa ? ldr<R>(a.kappa, k) : R(-1.0);
    land = a.inactive ? a.inactive[k] != 0 : false;
    if (P.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    else { c.du = c.ua - c.ui; c.dv = c.va - c.vi; }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = surface_atmosphere_temperature(P, c.Ta, c.qa);
    if (skin) {
        c.rho_a = air_density(P, c.Ta, c.pa, c.qa);
        c.cp_a = cp_m(P, c.qa);
        c.L_s = latent_heat_sublim(P, c.Ta);
    } else {
        c.rho_a = c.cp_a = c.L_s = R(0);
    }
}

// The flux epilogue (atmosphere_ocean_fluxes.jl:157-196).
template <class S, class R>
__device__ __forceinline__ void ao_store(const DevIface<R>& P, const AOArgs<S>& a, int64_t k,
                                         const CellConst<R>& c, bool land, R us, R ts, R qst, R Ts, int iters) {
    R ui = c.ui, vi = c.vi;
    if (land) {   // zero_interface_state (interface_states.jl:800-803)
        us = ts = qst = R(0);
        Ts = R(273.15);
        ui = vi = R(0);
    }
    R du, dv;
    if (P.vel_form == NESF_WIND_VELOCITY) { du = c.ua; dv = c.va; }
    else { du = c.ua - ui; dv = c.va - vi; }
    R dU = M<R>::sqrt(du * du + dv * dv);
    R tx = dU == R(0) ? R(0) : -(us * us) * du / dU;
    R ty = dU == R(0) ? R(0) : -(us * us) * dv / dU;
    R rho = air_density(P, c.Ta, c.pa, c.qa);
    R cp = cp_m(P, c.qa);
    R Lv = latent_heat_vapor(P, c.Ta);
    st(a.Qv, k, -rho * Lv * us * qst);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    st(a.Ts, k, Ts - P.off_ifc);
    st(a.us, k, us);
    st(a.ts, k, ts);
    st(a.qs, k, qst);
    if (a.iters) a.iters[k] = iters;
}

// A land cell's zero interface state (zero_interface_state, interface_states.jl:800-803)
// through ao_store's epilogue without its FP64 divisions and square root: with u* =
// theta* = q* = 0 every output is a zero whose sign follows the signs of the air density
// p / (R_m T), of cp_m, of L_v and of the wind components. The guards keep each factor
// finite and clear of the rounding that a contracted multiply-add could move (R_m's and
// the heat capacities' sums far from cancelling, the density's quotient within range),
// so the signs are ao_store's; other cells take ao_store. rho is replaced by +-1 of its
// sign, and the division by |dU| > 0 leaves a zero unchanged. FP32 fields decide in FP32
// (Pf: the parameters rounded to FP32) with margins ten times wider, which the FP32
// rounding of each factor stays far inside; FP64 operations and conversions run at 1/64
// of the FP32 rate, and land is a third of the grid.
template <class S>
__device__ __forceinline__ void ao_store_land(const DevIface<double>& P, const DevIface<float>& Pf, const AOArgs<S>& a,
                                              int64_t k, int iters) {
    if constexpr (sizeof(S) == sizeof(float)) {
        const float ua = a.ua[k], va = a.va[k], Ta = a.Ta[k], pa = a.pa[k], qa = a.qa[k];
        const float f = 1.0f + (Pf.eps - 1.0f) * qa;
        const float den = gas_constant_air(Pf, qa) * Ta;
        const float cp = cp_m(Pf, qa), Lv = latent_heat_vapor(Pf, Ta);
        const bool clear = fabsf(f) > 1e-5f * (1.0f + fabsf(Pf.eps - 1.0f) * fabsf(qa)) &&
                           fabsf(cp) > 1e-5f * (fabsf(Pf.cpd) + fabsf(Pf.cpv - Pf.cpd) * fabsf(qa)) &&
                           fabsf(Lv) > 1e-5f * (fabsf(Pf.Lv0) + fabsf(Pf.cpv - Pf.cpl) * fabsf(Ta - Pf.T0)) &&
                           fabsf(pa) > 1e-30f && fabsf(pa) < 1e30f && fabsf(den) > 1e-30f && fabsf(den) < 1e30f &&
                           fabsf(cp) < 1e30f && fabsf(Lv) < 1e30f && isfinite(ua) && isfinite(va);
        if (clear) {
            const float r = copysignf(1.0f, pa) * copysignf(1.0f, den);
            const float z = 0.0f;
            const bool calm = ua == 0.0f && va == 0.0f;
            const float tx = calm ? 0.0f : -(z * z) * ua;
            const float ty = calm ? 0.0f : -(z * z) * va;
            st(a.Qv, k, -r * Lv * z * z);
            st(a.QT, k, -r * cp * z * z);
            st(a.Jv, k, -r * z * z);
            st(a.tx, k, r * tx);
            st(a.ty, k, r * ty);
            st(a.Ts, k, (S)(273.15 - P.off_ifc));
            st(a.us, k, z);
            st(a.ts, k, z);
            st(a.qs, k, z);
            if (a.iters) a.iters[k] = iters;
            return;
        }
        CellConst<double> c;
        bool land;
        ao_load(P, a, k, false, c, land);
        ao_store<S, double>(P, a, k, c, true, 0.0, 0.0, 0.0, 273.15, iters);
        return;
    }
    const double ua = ld(a.ua, k), va = ld(a.va, k), Ta = ld(a.Ta, k), pa = ld(a.pa, k), qa = ld(a.qa, k);
    const double f = 1.0 + (P.eps - 1.0) * qa;
    const double den = gas_constant_air(P, qa) * Ta;
    const double cp = cp_m(P, qa), Lv = latent_heat_vapor(P, Ta);
    const bool clear = fabs(f) > 1e-6 * (1.0 + fabs(P.eps - 1.0) * fabs(qa)) &&
                       fabs(cp) > 1e-6 * (fabs(P.cpd) + fabs(P.cpv - P.cpd) * fabs(qa)) &&
                       fabs(Lv) > 1e-6 * (fabs(P.Lv0) + fabs(P.cpv - P.cpl) * fabs(Ta - P.T0)) &&
                       fabs(pa) > 1e-30 && fabs(pa) < 1e30 && fabs(den) > 1e-30 && fabs(den) < 1e30 &&
                       fabs(cp) < 1e30 && fabs(Lv) < 1e30 && isfinite(ua) && isfinite(va);
    if (!clear) {
        CellConst<double> c;
        bool land;
        ao_load(P, a, k, false, c, land);
        ao_store<S, double>(P, a, k, c, true, 0.0, 0.0, 0.0, 273.15, iters);
        return;
    }
    const double r = copysign(1.0, pa) * copysign(1.0, den);   // the sign of the air density
    const double z = 0.0;
    const bool calm = ua * ua + va * va == 0.0;                  // |dU| = 0 (surface at rest)
    const double tx = calm ? 0.0 : -(z * z) * ua;
    const double ty = calm ? 0.0 : -(z * z) * va;
    st(a.Qv, k, -r * Lv * z * z);
    st(a.QT, k, -r * cp * z * z);
    st(a.Jv, k, -r * z * z);
    st(a.tx, k, r * tx);
    st(a.ty, k, r * ty);
    st(a.Ts, k, 273.15 - P.off_ifc);
    st(a.us, k, z);
    st(a.ts, k, z);
    st(a.qs, k, z);
    if (a.iters) a.iters[k] = iters;
}

// The adaptive pass-1 prologue: the cell's FP32 inputs with FP64 only where
// differences cancel (ao_load's quantities, rounded to FP32).
template <class S, bool SKIN>
__device__ __forceinline__ void ao_load_fast(const DevIface<double>& P, const DevIface<float>& Pf, const AOArgs<S>& a,
                                             int64_t k, Fast32& f) {
    CellConst<float>& c = f.c;
    c.ua = ldf(a.ua, k); c.va = ldf(a.va, k); c.Ta = ldf(a.Ta, k); c.pa = ldf(a.pa, k); c.qa = ldf(a.qa, k);
    if (Pf.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    else {   // in FP64: u_a - u_i cancels where the air moves with the water
        c.du = (float)(ld(a.ua, k) - (ld(a.uo, k) + ld(a.uo, k + 1)) / 2);
        c.dv = (float)(ld(a.va, k) - (ld(a.vo, k) + ld(a.vo, k + a.L.sj)) / 2);
    }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    const double Ta = ld(a.Ta, k), qa = ld(a.qa, k), lift = lift_temperature(P, qa);
    f.tha = Ta + lift;
    c.tha = (float)f.tha;
    f.Ts0 = ld(a.To, k) + P.off_int;
    if (SKIN) {
        c.rho_a = air_density(Pf, c.Ta, c.pa, c.qa);
        c.cp_a = cp_m(Pf, c.qa);
        c.L_s = latent_heat_sublim(Pf, c.Ta);
        c.kappa = a.kappa ? ldf(a.kappa, k) : -1.0f;
        c.hi = c.hs = c.hc = c.Rth = 0.0f;
        f.anc = skin_anchor(P, f.tha, f.Ts0, ld(a.So, k), qa, ld(a.pa, k), ldz(a.sw, k), ldz(a.lw, k));
    } else {
        fast_surface(P, Pf, Ta, qa, ld(a.pa, k), lift, f.Ts0, f.s);
    }
}

// The cancelling differences of ao_load_fast in double-float, as the record the classify
// pass stores per work-list slot for the adaptive pass 1 (anchor_pack).
template <class S, bool SKIN>
__device__ __forceinline__ void ao_anchor_df(const DevIface<df>& P, const DevIface<float>& Pf, const AOArgs<S>& a,
                                             int64_t k, float (&v)[kAnchorFloats]) {
    float du = 0.0f, dv = 0.0f;
    if (Pf.vel_form != NESF_WIND_VELOCITY) {   // u_a - u_i cancels where the air moves with the water
        du = (float)(ldr<df>(a.ua, k) - (ldr<df>(a.uo, k) + ldr<df>(a.uo, k + 1)) / df(2));
        dv = (float)(ldr<df>(a.va, k) - (ldr<df>(a.vo, k) + ldr<df>(a.vo, k + a.L.sj)) / df(2));
    }
    const df Ta = ldr<df>(a.Ta, k), qa = ldr<df>(a.qa, k), lift = lift_temperature(P, qa);
    const df tha = Ta + lift, Ts0 = ldr<df>(a.To, k) + P.off_int;
    SurfaceConst<float> sc{};
    SkinAnchor<float> an{};
    if (SKIN) an = skin_anchor(P, tha, Ts0, ldr<df>(a.So, k), qa, ldr<df>(a.pa, k), ldzr<df>(a.sw, k), ldzr<df>(a.lw, k));
    else fast_surface(P, Pf, Ta, qa, ldr<df>(a.pa, k), lift, Ts0, sc);
    anchor_pack<SKIN>(sc, an, du, dv, tha, Ts0, v);
}

// ao_load_fast's FP32 part, after anchor_load has set the cancelling differences.
template <class S, bool SKIN>
__device__ __forceinline__ void ao_load_fp32(const DevIface<float>& Pf, const AOArgs<S>& a, int64_t k, Fast32& f) {
    CellConst<float>& c = f.c;
    c.ua = ldf(a.ua, k); c.va = ldf(a.va, k); c.Ta = ldf(a.Ta, k); c.pa = ldf(a.pa, k); c.qa = ldf(a.qa, k);
    if (Pf.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = (float)f.tha;
    if (SKIN) {
        c.rho_a = air_density(Pf, c.Ta, c.pa, c.qa);
        c.cp_a = cp_m(Pf, c.qa);
        c.L_s = latent_heat_sublim(Pf, c.Ta);
        c.kappa = a.kappa ? ldf(a.kappa, k) : -1.0f;
        c.hi = c.hs = c.hc = c.Rth = 0.0f;
    }
}

// The adaptive pass-1 epilogue (ao_store's fluxes in FP32; the interface
// temperature in FP64).
template <class S>
__device__ __forceinline__ void ao_store_fast(const DevIface<double>& P, const DevIface<float>& Pf,
                                              const AOArgs<S>& a, int64_t k, const Fast32& f, float us, float ts,
                                              float qst, double Ts, int iters) {
    float tx, ty;
    stress_fast(us, f.c.du, f.c.dv, tx, ty);
    float rho = air_density(Pf, f.c.Ta, f.c.pa, f.c.qa);
    float cp = cp_m(Pf, f.c.qa);
    float Lv = latent_heat_vapor(Pf, f.c.Ta);
    st(a.Qv, k, -rho * Lv * us * qst);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    st(a.Ts, k, Ts - P.off_ifc);
    st(a.us, k, us);
    st(a.ts, k, ts);
    st(a.qs, k, qst);
    if (a.iters) a.iters[k] = iters;
}

// Warm-start features of a cell in FP32 (the training samples use the same).
template <class S>
__device__ __forceinline__ mlp::Features ao_features(const DevIface<float>& P, const AOArgs<S>& a, int64_t k) {
    float ua = ldf(a.ua, k), va = ldf(a.va, k), Ta = ldf(a.Ta, k), pa = ldf(a.pa, k), qa = ldf(a.qa, k);
    float du = ua, dv = va;
    if (P.vel_form != NESF_WIND_VELOCITY) {
        du = ua - 0.5f * (ldf(a.uo, k) + ldf(a.uo, k + 1));
        dv = va - 0.5f * (ldf(a.vo, k) + ldf(a.vo, k + a.L.sj));
    }
    float tha = surface_atmosphere_temperature(P, Ta, qa);
    return mlp::warm_features(P, du * du + dv * dv, tha, ldf(a.To, k) + P.off_int, qa, pa);
}

// Pass 0: land cells get the zero interface state; the others are compacted into
// the member's work list by the sign class of their buoyancy flux (and, with a
// warm start, leave their network features at their work-list slot).
template <class S, bool ENS>
__global__ void __launch_bounds__(128) ao_classify_kernel(AOArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                          const DevIface<double>* __restrict__ P64s,
                                                          const DevIface<float>* __restrict__ P32s, WorkList wl,
                                                          float* feat, DevStats* stats, DevIface<df> Pd, float* anc) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    const int m = blockIdx.y;
    const DevIface<double>& P = ENS ? P64s[m] : P64;
    const DevIface<float>& Pf = ENS ? P32s[m] : P32;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool in = r < ring;
    int i = in ? (int)(r % nxr) : 0, j = in ? (int)(r / nxr) : 0;
    int64_t k = a.L.at(i, j) + (int64_t)m * a.member_stride;
    bool land = in && a.inactive ? a.inactive[k] != 0 : false;
    bool needs = P.stop_kind == NESF_STOP_CONVERGENCE;
    bool active = in && !land;
    bool stable = false;
    mlp::Features F;
    if (active) {
        if (feat) {
            // the bulk Richardson number of the features has the sign of the buoyancy flux
            F = ao_features(Pf, a, k);
            stable = F.f[0] > 0.0f;
        } else {
            float Ts = (float)(ld(a.To, k) + P.off_int);
            stable = stable_class(Pf, ldf(a.Ta, k), ldf(a.pa, k), ldf(a.qa, k), Ts);
        }
    }
    int64_t slot = worklist_push(wl, m, active, stable, (uint32_t)r);
    if (feat && slot >= 0) mlp::store_features(feat, slot, F);
    if (!ENS && anc && slot >= 0) {   // the adaptive pass 1's cancelling differences (one member)
        float v[kAnchorFloats];
        if (P.temp_form != NESF_BULK_TEMPERATURE) ao_anchor_df<S, true>(Pd, Pf, a, k, v);
        else ao_anchor_df<S, false>(Pd, Pf, a, k, v);
        anchor_store(anc, slot, v);
    }
    if (in && land) ao_store_land(P, Pf, a, k, needs ? 0 : P.maxiter);
    if (stats && in && land) stats_add(stats, true, false, 0, false, false, 0, false, false);
}

// One entry of pass 1: the w-th cell of member m's work list.
template <class S, int PREC, bool SKIN>
__device__ __forceinline__ void ao_cell(const AOArgs<S>& a, const DevIface<double>& Pd, const DevIface<float>& Pf,
                                        const SolveOpts& so, const WorkList& wl, const ReplayQueue& rq,
                                        const float* guess, DevStats* stats, int m, int64_t w) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    int64_t r = worklist_get(wl, m, w);
    if (r < 0) return;
    int i = (int)(r % nxr), j = (int)(r / nxr);
    int64_t k = a.L.at(i, j) + (int64_t)m * a.member_stride;
    const uint32_t id = (uint32_t)(m * ring + r);
    float xw[3];
    const float* warm = mlp::guess_at(guess, worklist_slot(wl, m, w), xw);
    bool needs = Pd.stop_kind == NESF_STOP_CONVERGENCE;
    if constexpr (PREC == NESF_F32_ADAPTIVE) {
        // FP32 sweep kept when quiet and well contracting; the other cells go to the
        // packed polish pass or, with fixed iteration counts, to the FP64 replay
        if (!needs) {
            replay_push(rq, true, id);
            polish_push(rq, false, id);
            if (stats) stats_add(stats, true, false, 0, false, false, 0, true, false);
            return;
        }
        Fast32 f;
        ao_load_fast<S, SKIN>(Pd, Pf, a, k, f);
        float x[4] = {1e-4f, 1e-4f, 1e-4f, SKIN ? f.anc.dTi : 0.0f};   // atmosphere_ocean_fluxes.jl:132
        float J[SKIN ? 4 : 3][SKIN ? 4 : 3];
        float rho;
        int f32it = 0, reason = -1;
        bool fallback = false;
        int outcome = sweep_fp32<SKIN, true>(Pf, f.c, f.s, f.anc, x, so, f32it, reason, J, rho, warm, &fallback);
        replay_push(rq, outcome == FAST_REPLAY, id);
        polish_push(rq, outcome == FAST_POLISH, id);
        if (outcome != FAST_SOLVED) {
            if (stats) {
                stats_add(stats, true, false, 0, false, false, 0, outcome == FAST_REPLAY, fallback);
                if (outcome == FAST_REPLAY) stats_replay_reason(stats, reason);
            }
            return;
        }
        ao_store_fast(Pd, Pf, a, k, f, x[0], x[1], x[2], SKIN ? f.tha + (double)x[3] : f.Ts0, f32it);
        if (stats) stats_add(stats, true, true, f32it, false, false, 0, false, fallback);
        return;
    }
    CellConst<double> c;
    bool land;
    ao_load(Pd, a, k, SKIN, c, land);
    double us = 1e-4, ts = 1e-4, qst = 1e-4;   // initial guess (atmosphere_ocean_fluxes.jl:132)
    SurfaceConst<double> s{};
    if (SKIN && PREC != NESF_PLAIN_F64 && needs) s.Ts = c.Ti;   // solve_fast reads only T_s of a skin state
    else surface_const(Pd, c, c.Ti, surface_specific_humidity(Pd, c.pa, c.Ti), s);
    int iters = 0, f64it = 0;
    bool nonconv = false, fallback = false;
    int outcome = FAST_SOLVED, reason = -1;
    if (PREC == NESF_PLAIN_F64 || !needs) {
        iters = solve_plain<SKIN>(Pd, c, s, us, ts, qst, nonconv);
    } else {
        int f32it;
        outcome = solve_fast<SKIN>(Pd, Pf, c, s, us, ts, qst, so, f32it, f64it, reason, warm, &fallback);
        iters = f32it + f64it;
    }
    if (PREC != NESF_PLAIN_F64) replay_push(rq, outcome == FAST_REPLAY, id);
    if (outcome != FAST_SOLVED) {
        if (stats) {
            stats_add(stats, true, false, 0, false, false, 0, outcome == FAST_REPLAY, fallback);
            if (outcome == FAST_REPLAY) stats_replay_reason(stats, reason);
        }
        return;
    }
    ao_store(Pd, a, k, c, false, us, ts, qst, s.Ts, iters);
    if (stats) stats_add(stats, true, true, iters, nonconv, f64it > 0, f64it, false, fallback);
}

// Pass 1: the compacted cells (unstable first, then stable), one thread each. With
// NESF_FETCH_OCEAN (FP32 solvers, one member) the grid is the resident blocks only and each
// warp takes the next 32 entries of the list (counter rq.count[kFetchCounter]) until it is
// exhausted: a warp that finishes early starts on new cells instead of holding its
// block's slot until the block's slowest warp is done. Each cell's arithmetic is the
// same under both schedules.
template <class S, int PREC, bool SKIN, bool ENS>
__global__ void __launch_bounds__(128, ENS ? 4 : (PREC == NESF_F32_ADAPTIVE ? 5 : 3)) ao_kernel(AOArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                              const DevIface<double>* __restrict__ P64s,
                                                              const DevIface<float>* __restrict__ P32s, SolveOpts so,
                                                              WorkList wl, ReplayQueue rq, const float* guess,
                                                              DevStats* stats) {
    const int m = blockIdx.y;
    __shared__ DevIface<double> sP64;
    __shared__ DevIface<float> sP32;
    if (ENS) {
        if (threadIdx.x == 0) {
            sP64 = P64s[m];
            sP32 = P32s[m];
        }
        __syncthreads();
    }
    const DevIface<double>& Pd = ENS ? sP64 : P64;
    const DevIface<float>& Pf = ENS ? sP32 : P32;
    const bool fetch = !ENS && PREC != NESF_PLAIN_F64 && (so.fetch & NESF_FETCH_OCEAN);
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (;;) {
        if (fetch) {
            unsigned base = 0;
            if ((threadIdx.x & 31) == 0) base = atomicAdd(&rq.count[kFetchCounter], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= wl.count[0] + wl.count[1]) return;
            w = (int64_t)base + (threadIdx.x & 31);
        }
        ao_cell<S, PREC, SKIN>(a, Pd, Pf, so, wl, rq, guess, stats, m, w);
        if (!fetch) return;
    }
}

// The atmosphere-ocean cell of the adaptive pass 1 (adaptive_pass1's adapter).
template <class S, bool SKIN>
struct AOAdaptiveCell {
    const AOArgs<S>& a;
    const DevIface<double>& P64;
    const DevIface<float>& P32;
    const float* anc;      // the classify pass's records (null: the FP64 prologue here)
    Fast32 f;
    int64_t k;
    uint32_t id;
    __device__ __forceinline__ void load(int64_t r, int64_t slot, float (&start)[4]) {
        const int nxr = a.L.nx + 2;
        const int i = (int)(r % nxr), j = (int)(r / nxr);
        k = a.L.at(i, j);
        id = (uint32_t)r;
        if (anc) {
            anchor_load<SKIN>(anc, slot, f);
            ao_load_fp32<S, SKIN>(P32, a, k, f);
        } else {
            ao_load_fast<S, SKIN>(P64, P32, a, k, f);
        }
        start[0] = start[1] = start[2] = 1e-4f;   // atmosphere_ocean_fluxes.jl:132
        start[3] = SKIN ? f.anc.dTi : 0.0f;
    }
    __device__ __forceinline__ void store(const float (&x)[4], int iters) {
        ao_store_fast(P64, P32, a, k, f, x[0], x[1], x[2], SKIN ? f.tha + (double)x[3] : f.Ts0, iters);
    }
};

// Pass 1 of the adaptive solver, one member, convergence stopping rule: adaptive_pass1
// with the schedule of SolveOpts::fetch / refill.
// Seven resident blocks per SM (72 registers) with a bulk interface temperature: its sweep
// state fits with few spills once the unused fourth state component is a constant and the
// cancelling differences come from the classify pass's records, and the extra warps hide
// more of its dependent latency (1/8-degree step: 1.32 ms at 5 blocks, 1.23 at 6 with the
// FP64 prologue; with the records 1.08 at 5, 1.03 at 6, 0.99 at 7); five with a skin
// temperature.
template <class S, bool SKIN>
__global__ void __launch_bounds__(128, SKIN ? NESF_ADAPTIVE_MIN_BLOCKS : NESF_ADAPTIVE_MIN_BLOCKS + 2) ao_adaptive_kernel(AOArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                             SolveOpts so, WorkList wl, ReplayQueue rq,
                                                             const float* guess, DevStats* stats, const float* anc) {
    AOAdaptiveCell<S, SKIN> cell{a, P64, P32, anc};
    adaptive_pass1<SKIN>(cell, P32, so, wl, rq, guess, stats, (so.fetch & NESF_FETCH_OCEAN) != 0);
}

// Pass 1b (ADAPTIVE): the cells whose FP32 result was not kept, packed, through
// pass 1's FP32 sweep + FP64 Newton polish; those that need it go on to the replay.
// R: the Newton steps' arithmetic, with the parameters Pr (or per member P64s): double, the
// drop-in's FP64 (the double-float instantiation measured slower than FP64 on these
// throughput passes).
template <class S, bool SKIN, class R = double>
__global__ void __launch_bounds__(128) ao_polish_kernel(AOArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                        DevIface<R> Pr, const DevIface<double>* __restrict__ P64s,
                                                        const DevIface<float>* __restrict__ P32s, SolveOpts so,
                                                        ReplayQueue rq, int rpart, DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    const unsigned n = rq.count[1];
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n && (int64_t)q < rq.capacity;
         q += gridDim.x * blockDim.x) {
        uint32_t id = rq.idx[rq.capacity + q];
        int64_t m = (int64_t)id / ring, r = (int64_t)id % ring;
        const DevIface<double>& P = P64s ? P64s[m] : P64;
        const DevIface<float>& Pf = P32s ? P32s[m] : P32;
        int i = (int)(r % nxr), j = (int)(r / nxr);
        int64_t k = a.L.at(i, j) + m * a.member_stride;
        // pass 1's sweep from the cold start (its inputs and its strict stopping rule),
        // then the FP64 Newton steps with the reference's FP64 cell constants
        Fast32 f;
        ao_load_fast<S, SKIN>(P, Pf, a, k, f);
        float x[4] = {1e-4f, 1e-4f, 1e-4f, SKIN ? f.anc.dTi : 0.0f};
        float J[SKIN ? 4 : 3][SKIN ? 4 : 3];
        float rho;
        int f32it = 0, f64it = 0, reason = -1;
        int outcome = sweep_fp32<SKIN, false, true>(Pf, f.c, f.s, f.anc, x, so, f32it, reason, J, rho, nullptr,
                                                    nullptr);
        const DevIface<R>& PR = member_params(Pr, P64s, m);
        CellConst<R> c;
        SurfaceConst<R> s{};
        R us = R(0), ts = R(0), qst = R(0);
        if (outcome != FAST_REPLAY) {
            bool land;
            ao_load(PR, a, k, SKIN, c, land);
            if (SKIN) s.Ts = c.Ti;
            else surface_const(PR, c, c.Ti, surface_specific_humidity(PR, c.pa, c.Ti), s);
            outcome = newton_fp64<SKIN, R>(PR, c, s, x, J, rho, so, us, ts, qst, f64it, reason);
        }
        replay_push(rq, outcome == FAST_REPLAY, id, rpart);
        if (outcome == FAST_REPLAY) {
            if (stats) {
                stats_add(stats, false, false, 0, false, false, 0, true, false);
                stats_replay_reason(stats, reason);
            }
            continue;
        }
        ao_store(PR, a, k, c, false, us, ts, qst, s.Ts, f32it + f64it);
        if (stats) stats_add(stats, false, true, f32it + f64it, false, true, f64it, false, false);
    }
}

// Pass 2: the cells queued in `part`, packed, through the reference's FP64 iteration, two
// lanes per cell (LanePair: the profiles' stability functions and logarithms split between them).
// R: double, or df for one member (the parameters in Pr; ensembles' members' parameters are FP64).
template <class S, bool SKIN, class R = double>
__global__ void __launch_bounds__(128) ao_replay_kernel(AOArgs<S> a, DevIface<R> Pr,
                                                        const DevIface<R>* __restrict__ Ps, ReplayQueue rq,
                                                        int part, DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    const unsigned n = rq.count[part];
    const LanePair lp{3u << ((threadIdx.x & 31u) & ~1u), (int)(threadIdx.x & 1u)};
    for (unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 1; q < n && (int64_t)q < rq.capacity;
         q += (gridDim.x * blockDim.x) >> 1) {
        uint32_t id = rq.idx[(int64_t)part * rq.capacity + q];
        int64_t m = (int64_t)id / ring, r = (int64_t)id % ring;
        const DevIface<R>& P = Ps ? Ps[m] : Pr;
        int i = (int)(r % nxr), j = (int)(r / nxr);
        int64_t k = a.L.at(i, j) + m * a.member_stride;
        CellConst<R> c;
        bool land;
        ao_load(P, a, k, SKIN, c, land);
        R us = R(1e-4), ts = R(1e-4), qst = R(1e-4);
        R qs0 = surface_specific_humidity(P, c.pa, c.Ti);
        SurfaceConst<R> s;
        surface_const(P, c, c.Ti, qs0, s);
        bool nonconv;
        int it = solve_plain<SKIN, false, true, R>(P, c, s, us, ts, qst, nonconv, lp);
        const bool mine = lp.half == 0;   // lane 0 of the pair stores and counts
        if (mine) ao_store(P, a, k, c, false, us, ts, qst, s.Ts, it);
        if (stats) stats_add(stats, false, mine, it, mine && nonconv, false, mine ? it : 0, false, false);
    }
}

template <class S>
static cudaError_t launch_ao_t(const AOArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                               const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec,
                               bool skin, SolveOpts so, const WorkList& wl, const ReplayQueue& rq,
                               const WarmStart& ws, DevStats* stats, cudaStream_t stream,
                               cudaEvent_t before_pass1, const TailLane* tail, MidHook* mid) {
    const int64_t ring = (int64_t)(a.L.nx + 2) * (a.L.ny + 2);
    const int threads = so.block;   // <= 128: the kernels are compiled with __launch_bounds__(128)
    const int nm = members > 1 ? members : 1;
    dim3 grid((unsigned)((ring + threads - 1) / threads), nm);
    bool ens = members > 1 || P64s != nullptr;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // warm start (FP32 modes, one member): features in pass 0, the network's guesses before pass 1
    const bool warm = ws.mlp != nullptr && prec != NESF_PLAIN_F64 && !ens && !skin &&
                      P64.flux_form == NESF_FLUXES_SIMILARITY_THEORY;   // the network predicts similarity theory
    float* feat = warm ? ws.feat : nullptr;
    const float* guess = warm ? ws.guess : nullptr;
    cudaError_t e = cudaMemsetAsync(wl.count, 0, sizeof(unsigned) * 2 * nm, stream);
    // rq.count: [0, 1] the deferred queues, [kFetchCounter] pass 1's fetch counter
    if (e == cudaSuccess && prec != NESF_PLAIN_F64)
        e = cudaMemsetAsync(rq.count, 0, kQueueCounters * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    // the adaptive pass 1 of one member under the convergence stopping rule loads its cancelling
    // differences from the classify pass's records (double-float) when the caller has a buffer
    const bool anchors = prec == NESF_F32_ADAPTIVE && so.fp32_rho > 0.0f && !ens &&
                         P64.stop_kind == NESF_STOP_CONVERGENCE && ws.anc && so.pdf;
    float* anc = anchors ? ws.anc : nullptr;
    if (ens)
        ao_classify_kernel<S, true><<<grid, threads, 0, stream>>>(a, P64, P32, P64s, P32s, wl, nullptr, stats,
                                                                  DevIface<df>{}, nullptr);
    else
        ao_classify_kernel<S, false><<<grid, threads, 0, stream>>>(a, P64, P32, P64s, P32s, wl, feat, stats,
                                                                   so.pdf ? *so.pdf : DevIface<df>{}, anc);
    trace_mark(so.tracer, "ao_classify", stream);
    if (warm) {
        e = mlp_pass((void*)ws.mlp, ws.feat, nullptr, ws.guess, 0, wl.count, wl.per_member, so.infer_per_sm * sms,
                     true, stream);
        if (e != cudaSuccess) return e;
        trace_mark(so.tracer, "ao_warm_start_inference", stream);
    }
    if (mid) {
        if (mid->ready && (e = cudaEventRecord(mid->ready, stream)) != cudaSuccess) return e;
        if (mid->fn && (mid->status = mid->fn(mid->arg)) != NESF_OK) return cudaErrorLaunchFailure;
    }
    if (before_pass1 && (e = cudaStreamWaitEvent(stream, before_pass1, 0)) != cudaSuccess) return e;
#define NESF_AO_LAUNCH(PR, SK, EN) \
    ao_kernel<S, PR, SK, EN><<<pass1_grid(ao_kernel<S, PR, SK, EN>, grid, threads, sms,                       \
                                          !EN && PR != NESF_PLAIN_F64 && (so.fetch & NESF_FETCH_OCEAN)),     \
                               threads, 0, stream>>>(a, P64, P32, P64s, P32s, so, wl, rq, guess, stats)
#define NESF_AO_ENS(PR, SK) \
    do { if (ens) NESF_AO_LAUNCH(PR, SK, true); else NESF_AO_LAUNCH(PR, SK, false); } while (0)
#define NESF_AO_SKIN(PR) \
    do { if (skin) NESF_AO_ENS(PR, true); else NESF_AO_ENS(PR, false); } while (0)
    // the adaptive pass 1 keeps FP32 results up to fp32_rho; fp32_rho = 0 keeps none: the
    // POLISH pass 1, which polishes every cell in place
    const bool adaptive = prec == NESF_F32_ADAPTIVE && so.fp32_rho > 0.0f;
    // the adaptive pass 1 of one member under the convergence stopping rule: every schedule in
    // one kernel (ao_adaptive_kernel)
    const bool one = adaptive && !ens && P64.stop_kind == NESF_STOP_CONVERGENCE;
    const bool fetch_ao = (so.fetch & NESF_FETCH_OCEAN) != 0;
    if (prec == NESF_PLAIN_F64) NESF_AO_SKIN(NESF_PLAIN_F64);
    else if (one && skin)
        ao_adaptive_kernel<S, true><<<pass1_grid(ao_adaptive_kernel<S, true>, grid, threads, sms, fetch_ao, so.cells), threads,
                                      0, stream>>>(a, P64, P32, so, wl, rq, guess, stats, anc);
    else if (one)
        ao_adaptive_kernel<S, false><<<pass1_grid(ao_adaptive_kernel<S, false>, grid, threads, sms, fetch_ao, so.cells),
                                       threads, 0, stream>>>(a, P64, P32, so, wl, rq, guess, stats, anc);
    else if (adaptive) NESF_AO_SKIN(NESF_F32_ADAPTIVE);
    else NESF_AO_SKIN(NESF_F32_POLISH);
#undef NESF_AO_SKIN
#undef NESF_AO_ENS
#undef NESF_AO_LAUNCH
    e = cudaGetLastError();
    trace_mark(so.tracer, "ao_pass1", stream);
    if (e != cudaSuccess || prec == NESF_PLAIN_F64) return e;
    // passes 1b and 2: enough resident blocks to sweep the queues (grid-stride)
    unsigned g2 = (unsigned)(sms * so.deferred_per_sm);
    const DevIface<double>* pm = ens ? P64s : nullptr;
    // with a second lane, pass 1's replays (part 0) run beside the polish pass, whose own
    // replays (part 2) follow it; without, the polish pass's replays join part 0
    const bool split = adaptive && tail && tail->stream;
    cudaStream_t rs = stream;
    // the replays of one member in double-float arithmetic when the caller provides its
    // parameters (so.pdf), else in FP64
    auto replay = [&](cudaStream_t st, int part) {
        if (so.pdf && !ens) {
            (void)launch_ao_replay_df(a, *so.pdf, rq, part, skin, stats, g2, st);
        } else {
            if (skin) ao_replay_kernel<S, true><<<g2, 128, 0, st>>>(a, P64, pm, rq, part, stats);
            else ao_replay_kernel<S, false><<<g2, 128, 0, st>>>(a, P64, pm, rq, part, stats);
        }
    };
    if (split) {
        if ((e = cudaEventRecord(tail->fork, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(tail->stream, tail->fork, 0)) != cudaSuccess) return e;
        rs = tail->stream;
        replay(rs, 0);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        trace_mark(so.tracer, "ao_replay", rs);
    }
    const int rpart = split ? 2 : 0;
    if (adaptive) {
        if (skin)
            ao_polish_kernel<S, true><<<g2, 128, 0, stream>>>(a, P64, P32, P64, pm, ens ? P32s : nullptr, so, rq, rpart, stats);
        else ao_polish_kernel<S, false><<<g2, 128, 0, stream>>>(a, P64, P32, P64, pm, ens ? P32s : nullptr, so, rq, rpart, stats);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        trace_mark(so.tracer, "ao_polish", stream);
    }
    replay(stream, rpart);
    trace_mark(so.tracer, split ? "ao_polish_replay" : "ao_replay", stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (split) {
        if ((e = cudaEventRecord(tail->join, rs)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, tail->join, 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class S>
static cudaError_t preload_ao_t() {
    const void* kernels[] = {
        (const void*)ao_classify_kernel<S, false>,
        (const void*)ao_kernel<S, NESF_PLAIN_F64, false, false>, (const void*)ao_kernel<S, NESF_PLAIN_F64, true, false>,
        (const void*)ao_kernel<S, NESF_F32_POLISH, false, false>, (const void*)ao_kernel<S, NESF_F32_POLISH, true, false>,
        (const void*)ao_kernel<S, NESF_F32_ADAPTIVE, false, false>,
        (const void*)ao_kernel<S, NESF_F32_ADAPTIVE, true, false>,
        (const void*)ao_adaptive_kernel<S, false>, (const void*)ao_adaptive_kernel<S, true>,
        (const void*)ao_polish_kernel<S, false>, (const void*)ao_polish_kernel<S, true>,
        (const void*)ao_replay_kernel<S, false>, (const void*)ao_replay_kernel<S, true>};
    for (const void* k : kernels) {
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, k);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The build compiles this file once per storage type (NESF_STORAGE = 64, then 32) and per
// part (NESF_DF_PART = 0: every kernel but the double-float replays, 1: those, whose
// inlined arithmetic takes the compiler longest), so that the parts compile in parallel;
// undefined builds everything.
template <class S>
static cudaError_t launch_ao_replay_df_t(const AOArgs<S>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                         bool skin, DevStats* stats, unsigned grid, cudaStream_t s) {
    if (skin) ao_replay_kernel<S, true, df><<<grid, 128, 0, s>>>(a, P, nullptr, rq, part, stats);
    else ao_replay_kernel<S, false, df><<<grid, 128, 0, s>>>(a, P, nullptr, rq, part, stats);
    return cudaGetLastError();
}

// Loads the double-float replays (under lazy module loading), for preload_ao_kernels.
template <class S>
static cudaError_t preload_ao_replay_df_t() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)ao_replay_kernel<S, false, df>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)ao_replay_kernel<S, true, df>);
    return e;
}
#if !defined(NESF_DF_PART) || NESF_DF_PART == 1
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
cudaError_t launch_ao_replay_df(const AOArgs<double>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                bool skin, DevStats* stats, unsigned grid, cudaStream_t s) {
    return launch_ao_replay_df_t(a, P, rq, part, skin, stats, grid, s);
}
cudaError_t preload_ao_replay_df(const AOArgs<double>*) { return preload_ao_replay_df_t<double>(); }
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
cudaError_t launch_ao_replay_df(const AOArgs<float>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                bool skin, DevStats* stats, unsigned grid, cudaStream_t s) {
    return launch_ao_replay_df_t(a, P, rq, part, skin, stats, grid, s);
}
cudaError_t preload_ao_replay_df(const AOArgs<float>*) { return preload_ao_replay_df_t<float>(); }
#endif
#endif
#if !defined(NESF_DF_PART) || NESF_DF_PART == 0
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
cudaError_t launch_ao(const AOArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t before_pass1, const TailLane* tail, MidHook* mid) {
    return launch_ao_t(a, P64, P32, P64s, P32s, members, prec, skin, so, wl, rq, ws, stats, stream, before_pass1,
                       tail, mid);
}
cudaError_t preload_ao_kernels(const AOArgs<double>* p) {
    cudaError_t e = preload_ao_t<double>();
    return e == cudaSuccess ? preload_ao_replay_df(p) : e;
}
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
cudaError_t launch_ao(const AOArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t before_pass1, const TailLane* tail, MidHook* mid) {
    return launch_ao_t(a, P64, P32, P64s, P32s, members, prec, skin, so, wl, rq, ws, stats, stream, before_pass1,
                       tail, mid);
}
cudaError_t preload_ao_kernels(const AOArgs<float>* p) {
    cudaError_t e = preload_ao_t<float>();
    return e == cudaSuccess ? preload_ao_replay_df(p) : e;
}
#endif
#endif

}  // namespace nesf

namespace nesf {

// Training samples of the warm-start network: the features of every ring cell
// (ring order) and the transfer coefficients of the solved state in the fields.
template <class S>
__global__ void __launch_bounds__(256) ao_samples_kernel(AOArgs<S> a, DevIface<float> P, float* feat, float* targ) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ring) return;
    int i = (int)(r % nxr), j = (int)(r / nxr);
    int64_t k = a.L.at(i, j);
    mlp::Features F = ao_features(P, a, k);
    mlp::store_features(feat, r, F);
    if (!targ) return;
    bool land = a.inactive ? a.inactive[k] != 0 : false;
    float us = ldf(a.us, k), ts = ldf(a.ts, k), qs = ldf(a.qs, k);
    float cu = us / F.U, ct = ts / F.dth, cq = qs / F.dq;
    int mask = 0;
    if (!land && isfinite(cu) && us > 0.0f) mask |= 1;
    if (!land && fabsf(F.dth) >= 0.05f && isfinite(ct)) mask |= 2;
    if (!land && fabsf(F.dq) >= 1e-5f && isfinite(cq)) mask |= 4;
    *(float4*)(targ + r * 4) = make_float4(mask & 1 ? cu : 0.0f, mask & 2 ? ct : 0.0f, mask & 4 ? cq : 0.0f,
                                           (float)mask);
}

template <class S>
cudaError_t launch_ao_samples(const AOArgs<S>& a, const DevIface<float>& P32, float* feat, float* targ,
                              cudaStream_t s) {
    const int64_t ring = (int64_t)(a.L.nx + 2) * (a.L.ny + 2);
    ao_samples_kernel<S><<<(unsigned)((ring + 255) / 256), 256, 0, s>>>(a, P32, feat, targ);
    return cudaGetLastError();
}
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
template cudaError_t launch_ao_samples<double>(const AOArgs<double>&, const DevIface<float>&, float*, float*,
                                               cudaStream_t);
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
template cudaError_t launch_ao_samples<float>(const AOArgs<float>&, const DevIface<float>&, float*, float*,
                                              cudaStream_t);
#endif

}  // namespace nesf
