// nesf_ai.cu -- atmosphere-sea-ice similarity-theory solve.
//
// _compute_atmosphere_sea_ice_interface_state! (InterfaceComputations/atmosphere_sea_ice_fluxes.jl:65-185)
//
// Same structure as the atmosphere-ocean kernel: one thread per cell over the
// halo ring, PLAIN or POLISH solve in pass 1, packed FP64 replays in pass 2. The
// interface temperature is a SkinTemperature over ice and snow, so the solver
// state carries T_s as a fourth component.
#include "nesf_solve.cuh"

namespace nesf {

// R: double (the reference's FP64 iteration) or df (the adaptive solver's replays).
template <class S, class R>
__device__ __forceinline__ void ai_load(const DevIface<R>& P, const AIArgs<S>& a, int64_t k,
                                        CellConst<R>& c, R& aleph, R& Ts0, bool& land) {
    c.ua = ldr<R>(a.ua, k); c.va = ldr<R>(a.va, k); c.Ta = ldr<R>(a.Ta, k); c.pa = ldr<R>(a.pa, k);
    c.qa = ldr<R>(a.qa, k);
    c.Ti = ldr<R>(a.To, k) + P.off_int;   // ocean below the ice (atmosphere_sea_ice_fluxes.jl:92-94)
    c.Si = ldr<R>(a.So, k);
    c.ui = R(0); c.vi = R(0);            // sea-ice velocities are not used (:97-98)
    c.hi = ldr<R>(a.hi, k);
    c.hs = ldzr<R>(a.hs, k);
    c.hc = ldr<R>(a.hc, k);
    c.Rth = conductive_resistance(P, c.hs, c.hi);
    aleph = ldr<R>(a.aleph, k);
    Ts0 = ldr<R>(a.Ts, k) + P.off_ifc;
    c.sw = ldzr<R>(a.sw, k);
    c.lw = ldzr<R>(a.lw, k);
    c.kappa = R(-1.0);
    land = a.inactive ? a.inactive[k] != 0 : false;
    if (P.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    else { c.du = c.ua - R(0.0); c.dv = c.va - R(0.0); }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = surface_atmosphere_temperature(P, c.Ta, c.qa);
    c.rho_a = air_density(P, c.Ta, c.pa, c.qa);
    c.cp_a = cp_m(P, c.qa);
    c.L_s = latent_heat_sublim(P, c.Ta);
}

// The flux epilogue (atmosphere_sea_ice_fluxes.jl:154-184).
template <class S, class R>
__device__ __forceinline__ void ai_store(const DevIface<R>& P, const AIArgs<S>& a, int64_t k,
                                         const CellConst<R>& c, R us, R ts, R qst, R Ts, int iters) {
    R du = c.du, dv = c.dv;
    R dU = M<R>::sqrt(du * du + dv * dv);
    R tx = dU == R(0) ? R(0) : -(us * us) * du / dU;
    R ty = dU == R(0) ? R(0) : -(us * us) * dv / dU;
    R rho = c.rho_a, cp = c.cp_a, Li = c.L_s;
    st(a.Qv, k, -rho * us * qst * Li);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    a.Ts[k] = (S)(Ts - P.off_ifc);
    if (a.iters) a.iters[k] = iters;
}

// The adaptive pass-1 prologue: ai_load's quantities in FP32, FP64 only where
// differences cancel (the anchors, or theta_a - T_s and q_a - q_s).
template <class S, bool SKIN>
__device__ __forceinline__ void ai_load_fast(const DevIface<double>& P, const DevIface<float>& Pf, const AIArgs<S>& a,
                                             int64_t k, Fast32& f) {
    CellConst<float>& c = f.c;
    c.ua = ldf(a.ua, k); c.va = ldf(a.va, k); c.Ta = ldf(a.Ta, k); c.pa = ldf(a.pa, k); c.qa = ldf(a.qa, k);
    c.du = c.ua; c.dv = c.va;            // sea-ice velocities are not used (:97-98)
    c.dU2 = c.du * c.du + c.dv * c.dv;
    const double Ta = ld(a.Ta, k), qa = ld(a.qa, k), lift = lift_temperature(P, qa);
    f.tha = Ta + lift;
    c.tha = (float)f.tha;
    c.rho_a = air_density(Pf, c.Ta, c.pa, c.qa);
    c.cp_a = cp_m(Pf, c.qa);
    c.L_s = latent_heat_sublim(Pf, c.Ta);
    f.Ts0 = ld(a.Ts, k) + P.off_ifc;
    if (SKIN) {
        c.hi = ldf(a.hi, k);
        c.hs = a.hs ? ldf(a.hs, k) : 0.0f;
        c.hc = ldf(a.hc, k);
        c.Rth = conductive_resistance(Pf, c.hs, c.hi);
        c.kappa = -1.0f;
        f.anc = skin_anchor(P, f.tha, ld(a.To, k) + P.off_int, ld(a.So, k), qa, ld(a.pa, k), ldz(a.sw, k),
                            ldz(a.lw, k));
    } else {
        fast_surface(P, Pf, Ta, qa, ld(a.pa, k), lift, f.Ts0, f.s);
    }
}

// The cancelling differences of ai_load_fast in double-float, as the record the classify
// pass stores per work-list slot for the adaptive pass 1 (anchor_pack).
template <class S, bool SKIN>
__device__ __forceinline__ void ai_anchor_df(const DevIface<df>& P, const DevIface<float>& Pf, const AIArgs<S>& a,
                                             int64_t k, float (&v)[kAnchorFloats]) {
    const df Ta = ldr<df>(a.Ta, k), qa = ldr<df>(a.qa, k), lift = lift_temperature(P, qa);
    const df tha = Ta + lift, Ts0 = ldr<df>(a.Ts, k) + P.off_ifc;
    SurfaceConst<float> sc{};
    SkinAnchor<float> an{};
    if (SKIN)
        an = skin_anchor(P, tha, ldr<df>(a.To, k) + P.off_int, ldr<df>(a.So, k), qa, ldr<df>(a.pa, k),
                         ldzr<df>(a.sw, k), ldzr<df>(a.lw, k));
    else
        fast_surface(P, Pf, Ta, qa, ldr<df>(a.pa, k), lift, Ts0, sc);
    anchor_pack<SKIN>(sc, an, 0.0f, 0.0f, tha, Ts0, v);
}

// ai_load_fast's FP32 part, after anchor_load has set the cancelling differences.
template <class S, bool SKIN>
__device__ __forceinline__ void ai_load_fp32(const DevIface<float>& Pf, const AIArgs<S>& a, int64_t k, Fast32& f) {
    CellConst<float>& c = f.c;
    c.ua = ldf(a.ua, k); c.va = ldf(a.va, k); c.Ta = ldf(a.Ta, k); c.pa = ldf(a.pa, k); c.qa = ldf(a.qa, k);
    c.du = c.ua; c.dv = c.va;            // sea-ice velocities are not used (:97-98)
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = (float)f.tha;
    c.rho_a = air_density(Pf, c.Ta, c.pa, c.qa);
    c.cp_a = cp_m(Pf, c.qa);
    c.L_s = latent_heat_sublim(Pf, c.Ta);
    if (SKIN) {
        c.hi = ldf(a.hi, k);
        c.hs = a.hs ? ldf(a.hs, k) : 0.0f;
        c.hc = ldf(a.hc, k);
        c.Rth = conductive_resistance(Pf, c.hs, c.hi);
        c.kappa = -1.0f;
    }
}

// The adaptive pass-1 epilogue (ai_store's fluxes in FP32; the interface
// temperature in FP64).
template <class S>
__device__ __forceinline__ void ai_store_fast(const DevIface<double>& P, const AIArgs<S>& a, int64_t k,
                                              const Fast32& f, float us, float ts, float qst, double Ts, int iters) {
    float tx, ty;
    stress_fast(us, f.c.du, f.c.dv, tx, ty);
    const float rho = f.c.rho_a;
    st(a.Qv, k, -rho * us * qst * f.c.L_s);
    st(a.QT, k, -rho * f.c.cp_a * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    a.Ts[k] = (S)(Ts - P.off_ifc);
    if (a.iters) a.iters[k] = iters;
}

template <bool SKIN, bool PAIR = false, class R = double>
__device__ __forceinline__ int ai_plain(const DevIface<R>& P, const CellConst<R>& c, R Ts0, R& us, R& ts, R& qst,
                                        R& Ts, bool& nonconv, LanePair lp = LanePair{0u, 0}) {
    R qs0 = surface_specific_humidity(P, c.pa, Ts0);
    SurfaceConst<R> s;
    surface_const(P, c, Ts0, qs0, s);
    us = ts = qst = R(1e-4);   // initial guess (atmosphere_sea_ice_fluxes.jl:127)
    int it = solve_plain<SKIN, false, PAIR, R>(P, c, s, us, ts, qst, nonconv, lp);
    Ts = s.Ts;
    return it;
}

// The zero interface state of an ice-free or land cell through the flux epilogue
// (atmosphere_sea_ice_fluxes.jl:141-142, 154-184) without its FP64 arithmetic: with
// u* = theta* = q* = 0 every flux is a signed zero, -0 for the heat and vapour fluxes
// (-rho u* ...) and the sign of -du for tau_x (likewise tau_y), +0 when dU = 0, given
// a positive finite air density; other cells take the full epilogue.
template <class S>
__device__ __forceinline__ void ai_store_zero(const DevIface<double>& P, const DevIface<float>& Pf,
                                              const AIArgs<S>& a, int64_t k) {
    double ua = ld(a.ua, k), va = ld(a.va, k);
    double Ti = ld(a.To, k) + P.off_int;
    float rho = air_density(Pf, ldf(a.Ta, k), ldf(a.pa, k), ldf(a.qa, k));
    if (!(rho > 0.0f && rho < 3.0e38f) || ua != ua || va != va) {
        CellConst<double> c;
        double aleph, Ts0;
        bool land;
        ai_load(P, a, k, c, aleph, Ts0, land);
        ai_store(P, a, k, c, 0.0, 0.0, 0.0, c.Ti, 0);
        return;
    }
    const bool calm = ua == 0.0 && va == 0.0;
    st(a.Qv, k, -0.0);
    st(a.QT, k, -0.0);
    st(a.Jv, k, -0.0);
    st(a.tx, k, calm ? 0.0 : copysign(0.0, -ua));
    st(a.ty, k, calm ? 0.0 : copysign(0.0, -va));
    a.Ts[k] = (S)(Ti - P.off_ifc);
    if (a.iters) a.iters[k] = 0;
}

// Pass 0: ice-free and land cells get the zero state with the ocean temperature
// (atmosphere_sea_ice_fluxes.jl:141-142); the others go to the work list, or, with
// calm2 > 0, those whose wind speed squared is below calm2 to the early replay (queue
// part 3): in calm air the reference's fixed point converges slowly (40 to 100
// iterations), the FP32 sweep's acceptance tests often send such a cell to the FP64
// replay anyway, and its replay, the longest chain of dependent FP64 iterations of the
// solve, can then start at once, beside pass 1, instead of after it.
template <class S>
__global__ void __launch_bounds__(128) ai_classify_kernel(AIArgs<S> a, DevIface<double> P, DevIface<float> Pf,
                                                          WorkList wl, ReplayQueue rq, float calm2, float* feat,
                                                          DevStats* stats, DevIface<df> Pd, float* anc) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool in = r < ring;
    int i = in ? (int)(r % nxr) : 0, j = in ? (int)(r / nxr) : 0;
    int64_t k = a.L.at(i, j);
    bool skip = false, active = false, stable = false;
    float Ta = 0.0f, pa = 0.0f, qa = 0.0f, Ts0 = 0.0f;
    if (in) {
        bool land = a.inactive ? a.inactive[k] != 0 : false;
        bool needs = P.stop_kind == NESF_STOP_CONVERGENCE;
        skip = (needs && land) || ld(a.aleph, k) == 0.0;
        active = !skip;
        if (active) {
            Ta = ldf(a.Ta, k); pa = ldf(a.pa, k); qa = ldf(a.qa, k);
            Ts0 = (float)(ld(a.Ts, k) + P.off_ifc);
            stable = stable_class(Pf, Ta, pa, qa, Ts0);
        }
    }
    bool calm = false;
    if (active && calm2 > 0.0f) {
        float ua = ldf(a.ua, k), va = ldf(a.va, k);
        calm = ua * ua + va * va < calm2;
    }
    queue_push(rq, 3, calm, (uint32_t)r);
    if (calm && stats) stats_add(stats, true, false, 0, false, false, 0, true, false);
    active = active && !calm;
    int64_t slot = worklist_push(wl, 0, active, stable, (uint32_t)r);
    if (feat && slot >= 0) {
        // warm-start features (FP32) from the state before the iteration
        float ua = ldf(a.ua, k), va = ldf(a.va, k);
        float tha = surface_atmosphere_temperature(Pf, Ta, qa);
        mlp::store_features(feat, slot, mlp::warm_features(Pf, ua * ua + va * va, tha, Ts0, qa, pa));
    }
    if (anc && slot >= 0) {   // the adaptive pass 1's cancelling differences
        float v[kAnchorFloats];
        if (P.temp_form != NESF_BULK_TEMPERATURE) ai_anchor_df<S, true>(Pd, Pf, a, k, v);
        else ai_anchor_df<S, false>(Pd, Pf, a, k, v);
        anchor_store(anc, slot, v);
    }
    if (skip) {
        ai_store_zero(P, Pf, a, k);
        if (stats) stats_add(stats, true, false, 0, false, false, 0, false, false);
    }
}

// One entry of pass 1: the w-th cell of the work list.
template <class S, int PREC, bool SKIN>
__device__ __forceinline__ void ai_cell(const AIArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                                        const SolveOpts& so, const WorkList& wl, const ReplayQueue& rq,
                                        const float* guess, DevStats* stats, int64_t w) {
    const int nxr = a.L.nx + 2;
    int64_t r = worklist_get(wl, 0, w);
    if (r < 0) return;
    float xw[3];
    const float* warm = mlp::guess_at(guess, worklist_slot(wl, 0, w), xw);
    int i = (int)(r % nxr), j = (int)(r / nxr);
    int64_t k = a.L.at(i, j);
    const DevIface<double>& P = P64;
    bool needs = P.stop_kind == NESF_STOP_CONVERGENCE;
    if constexpr (PREC == NESF_F32_ADAPTIVE) {
        // FP32 sweep kept when quiet and well contracting; the other cells go to the
        // packed polish pass or, with fixed iteration counts, to the FP64 replay
        if (!needs) {
            replay_push(rq, true, (uint32_t)r);
            polish_push(rq, false, (uint32_t)r);
            if (stats) stats_add(stats, true, false, 0, false, false, 0, true, false);
            return;
        }
        Fast32 f;
        ai_load_fast<S, SKIN>(P, P32, a, k, f);
        float x[4] = {1e-4f, 1e-4f, 1e-4f, SKIN ? (float)(f.Ts0 - f.tha) : 0.0f};   // :127
        float J[SKIN ? 4 : 3][SKIN ? 4 : 3];
        float rho;
        int f32it = 0, reason = -1;
        bool fallback = false;
        int outcome = sweep_fp32<SKIN, true>(P32, f.c, f.s, f.anc, x, so, f32it, reason, J, rho, warm, &fallback);
        replay_push(rq, outcome == FAST_REPLAY, (uint32_t)r);
        polish_push(rq, outcome == FAST_POLISH, (uint32_t)r);
        if (outcome != FAST_SOLVED) {
            if (stats) {
                stats_add(stats, true, false, 0, false, false, 0, outcome == FAST_REPLAY, fallback);
                if (outcome == FAST_REPLAY) stats_replay_reason(stats, reason);
            }
            return;
        }
        ai_store_fast(P, a, k, f, x[0], x[1], x[2], SKIN ? f.tha + (double)x[3] : f.Ts0, f32it);
        if (stats) stats_add(stats, true, true, f32it, false, false, 0, false, fallback);
        return;
    }
    CellConst<double> c;
    double aleph, Ts0;
    bool land;
    ai_load(P, a, k, c, aleph, Ts0, land);
    double us = 0, ts = 0, qst = 0, Ts = c.Ti;
    int iters = 0, f64it = 0;
    bool nonconv = false, fallback = false;
    int outcome = FAST_SOLVED, reason = -1;
    if (PREC == NESF_PLAIN_F64 || !needs) {
        iters = ai_plain<SKIN>(P, c, Ts0, us, ts, qst, Ts, nonconv);
    } else {
        SurfaceConst<double> s{};
        if (SKIN) s.Ts = Ts0;   // solve_fast reads only T_s of a skin state
        else surface_const(P, c, Ts0, surface_specific_humidity(P, c.pa, Ts0), s);
        us = ts = qst = 1e-4;
        int f32it;
        outcome = solve_fast<SKIN>(P, P32, c, s, us, ts, qst, so, f32it, f64it, reason, warm, &fallback);
        iters = f32it + f64it;
        Ts = s.Ts;
    }
    if (PREC != NESF_PLAIN_F64) replay_push(rq, outcome == FAST_REPLAY, (uint32_t)r);
    if (outcome != FAST_SOLVED) {
        if (stats) {
            stats_add(stats, true, false, 0, false, false, 0, outcome == FAST_REPLAY, fallback);
            if (outcome == FAST_REPLAY) stats_replay_reason(stats, reason);
        }
        return;
    }
    ai_store(P, a, k, c, us, ts, qst, Ts, iters);
    if (stats) stats_add(stats, true, true, iters, nonconv, f64it > 0, f64it, false, fallback);
}

// Pass 1: the compacted ice cells, one thread each; with NESF_FETCH_SEA_ICE (FP32 solvers) the
// resident blocks only, each warp taking the next 32 entries of the list (counter
// rq.count[kFetchCounter]) until it is exhausted, as in the atmosphere-ocean pass 1.
template <class S, int PREC, bool SKIN>
__global__ void __launch_bounds__(128, PREC == NESF_F32_ADAPTIVE ? 5 : 1) ai_kernel(AIArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                 SolveOpts so, WorkList wl, ReplayQueue rq, const float* guess,
                                                 DevStats* stats) {
    const bool fetch = PREC != NESF_PLAIN_F64 && (so.fetch & NESF_FETCH_SEA_ICE);
    int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (;;) {
        if (fetch) {
            unsigned base = 0;
            if ((threadIdx.x & 31) == 0) base = atomicAdd(&rq.count[kFetchCounter], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= wl.count[0] + wl.count[1]) return;
            w = (int64_t)base + (threadIdx.x & 31);
        }
        ai_cell<S, PREC, SKIN>(a, P64, P32, so, wl, rq, guess, stats, w);
        if (!fetch) return;
    }
}

// The atmosphere-sea-ice cell of the adaptive pass 1 (adaptive_pass1's adapter).
template <class S, bool SKIN>
struct AIAdaptiveCell {
    const AIArgs<S>& a;
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
            ai_load_fp32<S, SKIN>(P32, a, k, f);
        } else {
            ai_load_fast<S, SKIN>(P64, P32, a, k, f);
        }
        start[0] = start[1] = start[2] = 1e-4f;   // atmosphere_sea_ice_fluxes.jl:127
        start[3] = SKIN ? (float)(f.Ts0 - f.tha) : 0.0f;
    }
    __device__ __forceinline__ void store(const float (&x)[4], int iters) {
        ai_store_fast(P64, a, k, f, x[0], x[1], x[2], SKIN ? f.tha + (double)x[3] : f.Ts0, iters);
    }
};

// Pass 1 of the adaptive solver under the convergence stopping rule: adaptive_pass1 with the
// schedule of SolveOpts::fetch / refill. The skin-temperature instantiation (four real
// state components) runs 4 blocks per SM at up to 128 registers, without spills: with its
// cancelling differences loaded from the classify pass's records it measured faster so
// than at 5 blocks (96 registers, 190 bytes of spill stores) or 6 (80, 374 bytes).
template <class S, bool SKIN>
__global__ void __launch_bounds__(128, SKIN ? NESF_ADAPTIVE_MIN_BLOCKS - 1 : NESF_ADAPTIVE_MIN_BLOCKS) ai_adaptive_kernel(AIArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                             SolveOpts so, WorkList wl, ReplayQueue rq,
                                                             const float* guess, DevStats* stats, const float* anc) {
    AIAdaptiveCell<S, SKIN> cell{a, P64, P32, anc};
    adaptive_pass1<SKIN>(cell, P32, so, wl, rq, guess, stats, (so.fetch & NESF_FETCH_SEA_ICE) != 0);
}

// Pass 1b (ADAPTIVE): the cells whose FP32 result was not kept, packed, through pass
// 1's FP32 sweep + FP64 Newton polish; those that need it go on to the replay. The
// initial interface temperature is still in a.Ts: pass 1 did not write these cells.
// STATE: pass 1 left each entry's sweep state (rq.pstate; with a skin temperature).
// R: the Newton steps' arithmetic, with the parameters Pr (double, the drop-in's FP64; the
// double-float instantiation measured slower than FP64 on these throughput passes).
template <class S, bool SKIN, bool STATE, class R = double>
__global__ void __launch_bounds__(128) ai_polish_kernel(AIArgs<S> a, DevIface<double> P, DevIface<float> P32,
                                                        DevIface<R> Pr, SolveOpts so, ReplayQueue rq, int rpart,
                                                        DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const unsigned n = rq.count[1];
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n && (int64_t)q < rq.capacity;
         q += gridDim.x * blockDim.x) {
        uint32_t id = rq.idx[rq.capacity + q];
        int64_t r = id;
        int i = (int)(r % nxr), j = (int)(r / nxr);
        int64_t k = a.L.at(i, j);
        // pass 1's sweep: its state when pass 1 left it (a skin temperature), else the sweep
        // again (the same inputs, start and strict stopping rule: the same decisions); then
        // the FP64 Newton steps with the reference's FP64 cell constants
        float x[4];
        float J[SKIN ? 4 : 3][SKIN ? 4 : 3];
        float rho;
        int f32it = 0, f64it = 0, reason = -1, outcome;
        if constexpr (STATE) {
            polish_state_load(rq, (int64_t)q, x, J, rho, f32it);
            outcome = FAST_POLISH;
        } else {
            Fast32 f;
            ai_load_fast<S, SKIN>(P, P32, a, k, f);
            x[0] = x[1] = x[2] = 1e-4f;
            x[3] = SKIN ? (float)(f.Ts0 - f.tha) : 0.0f;
            outcome = sweep_fp32<SKIN, false, true>(P32, f.c, f.s, f.anc, x, so, f32it, reason, J, rho, nullptr,
                                                    nullptr);
        }
        CellConst<R> c;
        SurfaceConst<R> s{};
        R us = R(0), ts = R(0), qst = R(0);
        if (outcome != FAST_REPLAY) {
            R aleph, Ts0;
            bool land;
            ai_load(Pr, a, k, c, aleph, Ts0, land);
            if (SKIN) s.Ts = Ts0;
            else surface_const(Pr, c, Ts0, surface_specific_humidity(Pr, c.pa, Ts0), s);
            outcome = newton_fp64<SKIN, R>(Pr, c, s, x, J, rho, so, us, ts, qst, f64it, reason);
        }
        replay_push(rq, outcome == FAST_REPLAY, id, rpart);
        if (outcome == FAST_REPLAY) {
            if (stats) {
                stats_add(stats, false, false, 0, false, false, 0, true, false);
                stats_replay_reason(stats, reason);
            }
            continue;
        }
        ai_store(Pr, a, k, c, us, ts, qst, s.Ts, f32it + f64it);
        if (stats) stats_add(stats, false, true, f32it + f64it, false, true, f64it, false, false);
    }
}

// Pass 2: the queued cells, packed, through the reference's FP64 iteration, two lanes per
// cell (LanePair: the profiles' stability functions and logarithms split between them). The
// initial interface temperature is still in a.Ts: pass 1 did not write these cells.
template <class S, class R = double>
__global__ void __launch_bounds__(128) ai_replay_kernel(AIArgs<S> a, DevIface<R> P, ReplayQueue rq, int part,
                                                        DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const unsigned n = rq.count[part];
    const LanePair lp{3u << ((threadIdx.x & 31u) & ~1u), (int)(threadIdx.x & 1u)};
    for (unsigned q = (blockIdx.x * blockDim.x + threadIdx.x) >> 1; q < n && (int64_t)q < rq.capacity;
         q += (gridDim.x * blockDim.x) >> 1) {
        int64_t r = rq.idx[(int64_t)part * rq.capacity + q];
        int i = (int)(r % nxr), j = (int)(r / nxr);
        int64_t k = a.L.at(i, j);
        CellConst<R> c;
        R aleph, Ts0;
        bool land;
        ai_load(P, a, k, c, aleph, Ts0, land);
        R us, ts, qst, Ts;
        bool nonconv;
        int it = P.temp_form != NESF_BULK_TEMPERATURE
                     ? ai_plain<true, true, R>(P, c, Ts0, us, ts, qst, Ts, nonconv, lp)
                     : ai_plain<false, true, R>(P, c, Ts0, us, ts, qst, Ts, nonconv, lp);
        const bool mine = lp.half == 0;   // lane 0 of the pair stores and counts
        if (mine) ai_store(P, a, k, c, us, ts, qst, Ts, it);
        if (stats) stats_add(stats, false, mine, it, mine && nonconv, false, mine ? it : 0, false, false);
    }
}

template <class S>
static cudaError_t launch_ai_t(const AIArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                               SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws,
                               DevStats* stats, cudaStream_t stream, cudaEvent_t after_solve, const TailLane* tail,
                               const TailLane* early, cudaEvent_t before_pass1, MidHook* mid) {
    const int64_t ring = (int64_t)(a.L.nx + 2) * (a.L.ny + 2);
    const int block = so.block;   // <= 128: the kernels are compiled with __launch_bounds__(128)
    dim3 grid((unsigned)((ring + block - 1) / block));
    // the replays in double-float arithmetic when the caller provides the parameters (so.pdf),
    // else in FP64
    auto ai_replay = [&](unsigned g, cudaStream_t st, int part) {
        if (so.pdf) (void)launch_ai_replay_df(a, *so.pdf, rq, part, stats, g, st);
        else ai_replay_kernel<S><<<g, 128, 0, st>>>(a, P64, rq, part, stats);
    };
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the learned warm start serves the bulk interface temperature: with a skin temperature the
    // iteration count is set by the temperature's clamped steps, which the network does not predict
    const bool warm = ws.mlp != nullptr && prec != NESF_PLAIN_F64 && P64.temp_form == NESF_BULK_TEMPERATURE &&
                      P64.flux_form == NESF_FLUXES_SIMILARITY_THEORY;
    cudaError_t e = cudaMemsetAsync(wl.count, 0, sizeof(unsigned) * 2, stream);
    // rq.count: [0, 3] the deferred queues, [kFetchCounter] pass 1's fetch counter
    if (e == cudaSuccess && prec != NESF_PLAIN_F64)
        e = cudaMemsetAsync(rq.count, 0, kQueueCounters * sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    // calm cells straight to the FP64 replay (the adaptive solver under the convergence
    // stopping rule; the queue's part 3 holds them): on the early lane beside pass 1 when
    // there is one, else with pass 1's replays. The choice is the solver's, the lane only
    // the schedule: every tuning replays the same cells.
    const bool adaptive_conv = prec == NESF_F32_ADAPTIVE && so.fp32_rho > 0.0f && P64.stop_kind == NESF_STOP_CONVERGENCE;
    const bool calm = adaptive_conv && so.calm_wind > 0.0f;
    const bool early_lane = calm && early && early->stream;
    // the adaptive pass 1 under the convergence stopping rule loads its cancelling differences
    // from the classify pass's records (double-float) when the caller has a buffer
    const bool anchors = prec == NESF_F32_ADAPTIVE && so.fp32_rho > 0.0f && P64.stop_kind == NESF_STOP_CONVERGENCE &&
                         ws.anc && so.pdf;
    float* anc = anchors ? ws.anc : nullptr;
    ai_classify_kernel<S><<<grid, block, 0, stream>>>(a, P64, P32, wl, rq, calm ? so.calm_wind * so.calm_wind : 0.0f,
                                                      warm ? ws.feat : nullptr, stats,
                                                      so.pdf ? *so.pdf : DevIface<df>{}, anc);
    trace_mark(so.tracer, "ai_classify", stream);
    if (early_lane) {
        if ((e = cudaEventRecord(early->fork, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(early->stream, early->fork, 0)) != cudaSuccess) return e;
        ai_replay((unsigned)(sms * so.deferred_ice), early->stream, 3);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        trace_mark(so.tracer, "ai_calm_replay", early->stream);
    }
    if (warm) {
        e = mlp_pass((void*)ws.mlp, ws.feat, nullptr, ws.guess, 0, wl.count, wl.per_member, so.infer_per_sm * sms,
                     true, stream);
        if (e != cudaSuccess) return e;
        trace_mark(so.tracer, "ai_warm_start_inference", stream);
    }
    const float* guess = warm ? ws.guess : nullptr;
    if (before_pass1 && (e = cudaStreamWaitEvent(stream, before_pass1, 0)) != cudaSuccess) return e;
    // the adaptive pass 1 keeps FP32 results up to fp32_rho; fp32_rho = 0 keeps none: the
    // POLISH pass 1, which polishes every cell in place
    const bool adaptive = prec == NESF_F32_ADAPTIVE && so.fp32_rho > 0.0f;
    const bool skin = P64.temp_form != NESF_BULK_TEMPERATURE;
#define NESF_AI_LAUNCH(PR, SK, G)                                                                          \
    ai_kernel<S, PR, SK><<<pass1_grid(ai_kernel<S, PR, SK>, grid, block, sms, PR != NESF_PLAIN_F64 && (so.fetch & NESF_FETCH_SEA_ICE)), \
                           block, 0, stream>>>(a, P64, P32, so, wl, rq, G, stats)
#define NESF_AI_SKIN(PR, G) do { if (skin) NESF_AI_LAUNCH(PR, true, G); else NESF_AI_LAUNCH(PR, false, G); } while (0)
    // the adaptive pass 1 under the convergence stopping rule: every schedule in one kernel
    const bool one = adaptive && P64.stop_kind == NESF_STOP_CONVERGENCE;
    const bool fetch_ai = (so.fetch & NESF_FETCH_SEA_ICE) != 0;
    if (prec == NESF_PLAIN_F64) NESF_AI_SKIN(NESF_PLAIN_F64, nullptr);
    else if (one && skin)
        ai_adaptive_kernel<S, true><<<pass1_grid(ai_adaptive_kernel<S, true>, grid, block, sms, fetch_ai, so.cells), block, 0,
                                      stream>>>(a, P64, P32, so, wl, rq, guess, stats, anc);
    else if (one)
        ai_adaptive_kernel<S, false><<<pass1_grid(ai_adaptive_kernel<S, false>, grid, block, sms, fetch_ai, so.cells), block,
                                       0, stream>>>(a, P64, P32, so, wl, rq, guess, stats, anc);
    else if (adaptive) NESF_AI_SKIN(NESF_F32_ADAPTIVE, guess);
    else NESF_AI_SKIN(NESF_F32_POLISH, guess);
#undef NESF_AI_SKIN
#undef NESF_AI_LAUNCH
    e = cudaGetLastError();
    trace_mark(so.tracer, "ai_pass1", stream);
    if (e == cudaSuccess && after_solve) e = cudaEventRecord(after_solve, stream);
    if (e == cudaSuccess && mid && mid->fn && (mid->status = mid->fn(mid->arg)) != NESF_OK) return cudaErrorLaunchFailure;
    if (e != cudaSuccess || prec == NESF_PLAIN_F64) return e;
    const unsigned g2 = (unsigned)(sms * so.deferred_ice);
    if (!adaptive) {
        ai_replay(g2, stream, 0);
        trace_mark(so.tracer, "ai_replay", stream);
        return cudaGetLastError();
    }

    // pass 1's replays (part 0) beside the polish pass, whose own replays (part 2) follow it
    cudaStream_t rs = stream;
    if (tail && tail->stream) {
        if ((e = cudaEventRecord(tail->fork, stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(tail->stream, tail->fork, 0)) != cudaSuccess) return e;
        rs = tail->stream;
    }
    ai_replay(g2, rs, 0);
    trace_mark(so.tracer, "ai_replay", rs);
    if (calm && !early_lane) {
        ai_replay(g2, rs, 3);
        trace_mark(so.tracer, "ai_calm_replay", rs);
    }
    if (mid && mid->wait && (e = cudaStreamWaitEvent(stream, mid->wait, 0)) != cudaSuccess) return e;
    if (skin && rq.pstate) ai_polish_kernel<S, true, true><<<g2, 128, 0, stream>>>(a, P64, P32, P64, so, rq, 2, stats);
    else if (skin) ai_polish_kernel<S, true, false><<<g2, 128, 0, stream>>>(a, P64, P32, P64, so, rq, 2, stats);
    else ai_polish_kernel<S, false, false><<<g2, 128, 0, stream>>>(a, P64, P32, P64, so, rq, 2, stats);
    trace_mark(so.tracer, "ai_polish", stream);
    ai_replay(g2, stream, 2);
    trace_mark(so.tracer, "ai_polish_replay", stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (rs != stream) {
        if ((e = cudaEventRecord(tail->join, rs)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, tail->join, 0)) != cudaSuccess) return e;
    }
    if (early_lane) {   // the early lane (only on this path: calm needs the adaptive solver) joins last
        if ((e = cudaEventRecord(early->join, early->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, early->join, 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The build compiles this file once per storage type (NESF_STORAGE = 64, then 32) and per
// part (NESF_DF_PART = 0: every kernel but the double-float replay, 1: that one, whose
// inlined arithmetic takes the compiler longest), so that the parts compile in parallel;
// undefined builds everything.
#if !defined(NESF_DF_PART) || NESF_DF_PART == 1
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
cudaError_t launch_ai_replay_df(const AIArgs<double>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                DevStats* stats, unsigned grid, cudaStream_t s) {
    ai_replay_kernel<double, df><<<grid, 128, 0, s>>>(a, P, rq, part, stats);
    return cudaGetLastError();
}
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
cudaError_t launch_ai_replay_df(const AIArgs<float>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                DevStats* stats, unsigned grid, cudaStream_t s) {
    ai_replay_kernel<float, df><<<grid, 128, 0, s>>>(a, P, rq, part, stats);
    return cudaGetLastError();
}
#endif
#endif
#if !defined(NESF_DF_PART) || NESF_DF_PART == 0
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
cudaError_t launch_ai(const AIArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t after_solve, const TailLane* tail, const TailLane* early,
                      cudaEvent_t before_pass1, MidHook* mid) {
    return launch_ai_t(a, P64, P32, prec, so, wl, rq, ws, stats, stream, after_solve, tail, early, before_pass1, mid);
}
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
cudaError_t launch_ai(const AIArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t after_solve, const TailLane* tail, const TailLane* early,
                      cudaEvent_t before_pass1, MidHook* mid) {
    return launch_ai_t(a, P64, P32, prec, so, wl, rq, ws, stats, stream, after_solve, tail, early, before_pass1, mid);
}
#endif
#endif

}  // namespace nesf
