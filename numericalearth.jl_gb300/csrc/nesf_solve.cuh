// nesf_solve.cuh -- the per-cell solvers shared by the atmosphere-ocean and
// atmosphere-sea-ice kernels, and their argument bundles.
//
// PLAIN   compute_interface_state with the reference's FP64 fixed point
//         (InterfaceComputations/compute_interface_state.jl:10-58).
// POLISH  the same fixed point in FP32 from the same start until it converges or
//         stalls at FP32 resolution, then FP64 Newton steps on x = F(x) (J from
//         FP32 finite differences, the residual from one FP64 evaluation of F).
//         Cells whose result could legitimately differ from the reference's by
//         more than `path_tol` -- because the reference's absolute stopping rule
//         leaves that much room there -- are queued for a replay of the
//         reference's FP64 iteration from the start, which a second, packed
//         kernel runs. Replaying them in place would idle the other 31 lanes.
// ADAPTIVE POLISH, except that a cell keeps its FP32 result when every state
//         component converged at FP32 resolution and F contracts by at most
//         `fp32_rho`: the scales then carry the FP32 evaluation error (a few ulps,
//         the differences that cancel being anchored in FP64, see the delta form
//         below) amplified by 1 / (1 - rho). The other cells are queued for a
//         packed pass that polishes them in FP64.
#pragma once

#include "nesf_kernels.cuh"
#include "nesf_mlp.cuh"

namespace nesf {

// Kernel-boundary tracing (nesf_trace_enable): a host-side hook that the
// launchers call after each launch, recording an event on its stream; null when
// tracing is off.
struct Tracer {
    void (*mark)(void* self, const char* name, cudaStream_t s);
    void* self;
};

inline void trace_mark(const Tracer* t, const char* name, cudaStream_t s) {
    if (t && t->mark) t->mark(t->self, name, s);
}

// Knobs of the FP32 + FP64-polish solver.
enum { NESF_FETCH_OCEAN = 1, NESF_FETCH_SEA_ICE = 2 };

struct SolveOpts {
    int polish_steps;      // FP64 Newton steps
    float path_tol;        // replay threshold on the reference's stopping-error bound
    float fp32_rho;        // ADAPTIVE: keep the FP32 result below this contraction (0: never)
    float fallback_ratio;  // warm start: cold start when the first residual exceeds this times the cold one
    // launch shapes (host side; the autotuner's choice): threads per block of pass 1,
    // blocks per SM of the packed polish/replay passes and of the warm-start inference
    int block, deferred_per_sm, infer_per_sm;
    int fetch;             // pass 1 of the FP32 solvers where resident warps take 32 work-list entries
                           // at a time: NESF_FETCH_OCEAN | NESF_FETCH_SEA_ICE bits
    int refill;            // adaptive pass 1 with warp fetching: lanes idle before a warp takes new
                           // entries for them (32: all, the warp fetching; fewer: lane refill)
    const Tracer* tracer;  // host side: kernel-boundary trace (null: off)
    float calm_wind;       // adaptive sea-ice solve with an early lane: wind speed below which the
                           // classify pass sends a cell straight to the FP64 replay (0: none)
    int deferred_ice;      // blocks per SM of the sea-ice solve's packed polish and replay passes
    int cells;             // adaptive pass 1: work-list entries a thread takes in turn (one thread per
                           // entry: the grid shrinks by this factor) or a lane reserves per fetch
    const DevIface<df>* pdf;   // host side: the parameters in double-float, for the deferred passes
                               // of one member (null: FP64)
};

// Warm start of a solve: features written by the classify pass at the work-list
// slots, the network's guesses (u*, theta*, q*, valid) at the same slots.
struct WarmStart {
    float* feat;           // 8 floats per slot
    float* guess;          // 4 floats per slot
    const void* mlp;       // trained network (null: cold start)
    float* anc;            // adaptive one-member solves: the cancelling differences of each work-list
                           // slot (kAnchorFloats), written by the classify pass (null: pass 1 computes them)
};

// Active cells of one solve, compacted and split by the sign of the surface
// buoyancy flux so that a warp evaluates one branch of the stability functions.
// Member m owns idx[m * per_member, (m + 1) * per_member): unstable cells from the
// front, stable cells from the back; count[2m] and count[2m + 1] are their numbers.
struct WorkList {
    uint32_t* idx;
    unsigned int* count;
    int64_t per_member;
};

// Cells deferred to the packed passes, in parts of `capacity` entries: part 0 the
// cells to replay in FP64, part 1 the cells to polish (ADAPTIVE), part 2 (the
// sea-ice solve's, which replays the polish pass's cells apart so that the replay
// of pass 1's cells runs beside the polish pass) the polish pass's replays, part 3
// (the sea-ice solve's) the calm cells its classify pass sends straight to the
// replay (SolveOpts::calm_wind); count[part] are their numbers (zeroed before the
// solve), and count[kFetchCounter] is pass 1's fetch counter (SolveOpts::fetch). A
// cell that the polish pass sends on to a replay holds one entry in each of two parts.
constexpr int kFetchCounter = 4;

// Blocks of 128 threads per SM that the adaptive pass-1 kernels are compiled for (their
// register budget: 65536 / (128 x this), rounded down to a multiple of 8).
#ifndef NESF_ADAPTIVE_MIN_BLOCKS
#define NESF_ADAPTIVE_MIN_BLOCKS 5
#endif
constexpr int kQueueCounters = 5;
struct ReplayQueue {
    uint32_t* idx;          // linear cell ids (member * ring + ring index)
    unsigned int* count;
    int64_t capacity;
    float* pstate;          // pass 1's state of each part-1 entry (null: the polish pass repeats
                            // pass 1's sweep); kPolishStateFloats floats per entry
};

// Pass 1's state of a cell it sends to the polish pass (the adaptive solver with a skin
// temperature, whose pass 1 takes the central-difference Jacobian before its decisions, as
// the polish pass's own sweep does): the FP32 fixed point x, the Jacobian J (4 x 4), the
// contraction bound and the FP32 map evaluations, at the cell's polish-queue position, so
// that the polish pass goes straight to its FP64 Newton steps instead of repeating the
// sweep. Six float4 per entry.
constexpr int kPolishStateFloats = 24;

// A second stream for the deferred passes and its fork/join events (null: serial).
struct TailLane {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};

template <class S> struct AOArgs {
    Layout2 L;
    int64_t member_stride;
    const S *ua, *va, *Ta, *pa, *qa, *uo, *vo, *To, *So;
    const uint8_t* inactive;
    const S *sw, *lw, *kappa;
    S *Qv, *QT, *Jv, *tx, *ty, *us, *ts, *qs, *Ts;
    int32_t* iters;
};

template <class S> struct ALArgs {
    Layout2 L;
    const S *ua, *va, *Ta, *pa, *qa, *T, *sat;
    S *Qv, *QT, *Jv, *tx, *ty, *us, *ts, *qs, *Ts;
    int32_t* iters;
};

template <class S> struct AIArgs {
    Layout2 L;
    const S *ua, *va, *Ta, *pa, *qa, *To, *So, *hi, *hs, *hc, *aleph;
    const uint8_t* inactive;
    const S *sw, *lw;
    S* Ts;   // in/out
    S *Qv, *QT, *Jv, *tx, *ty;
    int32_t* iters;
};

// ---------------------------------------------------------------- FP32 sweep
// What the FP32 sweep learned about the reference's convergence: the drift
// vector of the last iteration that was still well above FP32 noise and the
// contraction rate between that drift and the one before it.
struct SweepTrace {
    float d[3];     // drift components (u*, theta*, q*)
    float lam;      // |d_k|_1 / |d_(k-1)|_1
};

template <class R, class Q>
__device__ __forceinline__ void convert_const(const CellConst<R>& a, CellConst<Q>& b) {
    b.ua = Q(a.ua); b.va = Q(a.va); b.Ta = Q(a.Ta); b.pa = Q(a.pa); b.qa = Q(a.qa);
    b.ui = Q(a.ui); b.vi = Q(a.vi); b.Ti = Q(a.Ti); b.Si = Q(a.Si);
    b.hi = Q(a.hi); b.hs = Q(a.hs); b.hc = Q(a.hc); b.sw = Q(a.sw); b.lw = Q(a.lw); b.kappa = Q(a.kappa);
    b.du = Q(a.du); b.dv = Q(a.dv); b.dU2 = Q(a.dU2); b.tha = Q(a.tha);
    b.rho_a = Q(a.rho_a); b.cp_a = Q(a.cp_a); b.L_s = Q(a.L_s); b.Rth = Q(a.Rth); b.qres = Q(a.qres);
}

template <class R, class Q>
__device__ __forceinline__ void convert_surface(const SurfaceConst<R>& a, SurfaceConst<Q>& b) {
    b.Ts = Q(a.Ts); b.qs = Q(a.qs); b.dth = Q(a.dth); b.dq = Q(a.dq);
    b.gTv = Q(a.gTv); b.A1 = Q(a.A1); b.A2 = Q(a.A2);
    b.nu_u = Q(a.nu_u); b.nu_t = Q(a.nu_t); b.nu_q = Q(a.nu_q);
}

// ------------------------------------------------ FP32 skin map in delta form
// The FP32 sweep of a skin temperature carries tau = T_s - theta_a instead of
// T_s. theta_a - T_s nearly cancels where the surface is close to the air
// temperature, and an FP32 T_s resolves only ~1.5e-5 K at 270 K: carried as tau,
// dtheta = -tau keeps FP32's relative precision. The other differences that
// cancel are anchored the same way, in FP64 once per cell: q_a - q_s(T_s) as
// (q_a - q_s(theta_a)) - (q_s(T_s) - q_s(theta_a)), the second term from the
// Clausius-Clapeyron ratio e_sat(T_s) / e_sat(theta_a) (log1p / expm1 of a small
// argument); and the net surface flux Q_v + I_up + Q_d as (I_up(theta_a) + Q_d)
// + (I_up(T_s) - I_up(theta_a)) + Q_v, I_up(T_s) - I_up(theta_a) from
// (1 + tau / theta_a)^4 - 1. The map is the reference's map; only its rounding
// differs. The FP64 polish and replay evaluate the reference's form.
template <class R> struct SkinAnchor {
    R dTi, dTb, dTm;   // interior, conductive-base and melting temperatures minus theta_a
    R pva, qsa, dqa;   // x e_sat(theta_a), q_s(theta_a) (no saturation cap), q_a - q_s(theta_a)
    R Qa0, Iupa;       // I_up(theta_a) + Q_d, I_up(theta_a) = sigma eps theta_a^4
    R gA, gK;          // ln e_sat(T) = gA ln T - gK / T + const
};

// The anchors of a cell from theta_a and the interior temperature in A, FP64 or double-float
// (the other inputs need no more than FP32's relative precision).
template <class A>
__device__ __forceinline__ SkinAnchor<float> skin_anchor(const DevIface<A>& P, A tha, A Ti, A Si, A qa, A pa, A sw,
                                                         A lw) {
    SkinAnchor<float> a;
    a.dTi = (float)(Ti - tha);
    A Tb = P.Tfw - P.slope * Si;
    Tb = Tb + P.off_ifc;
    a.dTb = (float)(Tb - tha);
    a.dTm = (float)(P.Tfw + P.off_ifc - tha);
    A pv = P.x * esat_exp(P, tha);
    A qsa = P.einv * pv / (pa - (A(1.0) - P.einv) * pv);
    a.pva = (float)pv;
    a.qsa = (float)qsa;
    a.dqa = (float)(qa - qsa);
    A sigma = P.has_rad ? P.sigma : A(0.0), eps = P.has_rad ? P.emis : A(0.0);
    A alb = P.has_rad ? P.alb : A(0.0), SW = P.has_rad ? sw : A(0.0), LW = P.has_rad ? lw : A(0.0);
    A T2 = tha * tha;
    A Iup = sigma * eps * (T2 * T2);
    A Qd = -(A(1.0) - alb) * SW - eps * LW;
    a.Iupa = (float)Iup;
    a.Qa0 = (float)(Iup + Qd);
    a.gA = (float)P.esA;
    a.gK = (float)P.esK;
    return a;
}

// flux_balance_temperature (interface_states.jl:434-457 diffusive, 468-524
// conductive) + the clamps of compute_interface_temperature, as tau -> tau'.
// `cond` (optional) receives the condition number of the update: the sum of the
// magnitudes of the terms that make up T_st - theta_a over the magnitude of their
// sum (1 where T_s is pinned), by which FP32 rounding of the terms is amplified.
template <class R>
__device__ __forceinline__ R skin_tau(const DevIface<R>& P, const CellConst<R>& c, const SkinAnchor<R>& A, R tau,
                                      R us, R ts, R qst, R* cond = nullptr) {
    R r = tau / c.tha;
    R dI = A.Iupa * (r * (R(4) + r * (R(6) + r * (R(4) + r))));   // I_up(T_s) - I_up(theta_a)
    R QT = -c.rho_a * c.cp_a * us * ts;
    R Qv = -c.rho_a * c.L_s * us * qst;
    R Qa = A.Qa0 + dI + Qv;
    R dT = -tau;                                                    // theta_a - T_s
    if (P.temp_form == NESF_SKIN_TEMPERATURE_DIFFUSIVE) {
        R kap = c.kappa >= R(0) ? M<R>::fmax(c.kappa, P.kap_diff) : P.kap_diff;
        R del = P.del_diff;
        R lam = R(1) / (P.rho_i * P.c_i);
        R JT = Qa * lam;
        R OmT = QT * lam;
        R D = kap * dT - OmT * del;
        R n1 = A.dTi * kap * dT, n2 = JT * dT * del;
        R tst = (n1 - n2) / D;                                       // T_st - theta_a
        tst = D == R(0) ? tau : tst;
        R dev = tst - A.dTi;
        if (cond) {
            R qa_mag = (fabs(A.Qa0) + fabs(dI) + fabs(Qv)) / fmax(fabs(Qa), R(1e-30));
            *cond = fabs(dev) > P.max_dT ? R(1) : (fabs(n1) + fabs(n2) * qa_mag) / fmax(fabs(n1 - n2), R(1e-30));
        }
        return A.dTi + clampr(dev, -P.max_dT, P.max_dT);
    }
    R Rth = c.Rth;
    R Om = dT == R(0) ? R(0) : QT / dT;
    R beta = R(4) * (A.Iupa + dI) / (c.tha + tau);
    R D = R(1) + beta * Rth - Om * Rth;
    R n2 = beta * Rth * tau;
    R tst = (A.dTb + n2 - Qa * Rth) / D;
    tst = D == R(0) ? tau : tst;
    tst = isnan(tst) ? tau : tst;
    R tp = tau + clampr(tst - tau, -P.max_dT, P.max_dT);
    bool free = tp < A.dTm && c.hi >= c.hc;
    if (cond) {
        R mag = fabs(A.dTb) + fabs(n2) + Rth * (fabs(A.Qa0) + fabs(dI) + fabs(Qv));
        *cond = free ? mag / fmax(fabs(A.dTb + n2 - Qa * Rth), R(1e-30)) : R(1);
    }
    tp = M<R>::fmin(tp, A.dTm);
    return c.hi >= c.hc ? tp : A.dTb;
}

// One FP32 application of F to (u*, theta*, q*, tau) (iterate_interface_state).
// `cond` (optional) receives the larger condition number of the two anchored
// differences, q_a - q_s and the temperature update.
template <class R>
__device__ __forceinline__ void iterate_skin_delta(const DevIface<R>& P, const CellConst<R>& c,
                                                   const SkinAnchor<R>& A, R& us, R& ts, R& qst, R& tau,
                                                   R* cond = nullptr) {
    R t1 = skin_tau(P, c, A, tau, us, ts, qst, cond);
    R T = c.tha + t1;
    R g = A.gA * log1pf(t1 / c.tha) + A.gK * t1 / (c.tha * T);    // ln e_sat(T) - ln e_sat(theta_a)
    R dpv = A.pva * expm1f(g);
    R pv = A.pva + dpv;
    R c2 = R(1) - P.einv;
    SurfaceConst<R> s;
    if (!(pv > R(0.999) * c.pa)) {
        R dqs = P.einv * c.pa * dpv / ((c.pa - c2 * pv) * (c.pa - c2 * A.pva));   // q_s(T) - q_s(theta_a)
        s.qs = A.qsa + dqs;
        s.dq = A.dqa - dqs;
        if (cond) *cond = fmax(*cond, (fabs(A.dqa) + fabs(dqs)) / fmax(fabs(s.dq), R(1e-30)));
    } else {
        R pvc = R(0.999) * c.pa;   // the saturation cap of surface_specific_humidity
        s.qs = P.einv * pvc / (c.pa - c2 * pvc);
        s.dq = c.qa - s.qs;
    }
    s.Ts = T;
    s.dth = -t1;
    R Tv = virtual_temperature(P, T, s.qs);
    R delta = P.eps - R(1);
    s.gTv = P.g / Tv;
    s.A1 = R(1) + delta * s.qs;
    s.A2 = delta * Tv;
    s.nu_u = air_viscosity(P.rough[0], T);
    s.nu_t = air_viscosity(P.rough[1], T);
    s.nu_q = air_viscosity(P.rough[2], T);
    R a, b, d;
    iterate_fluxes(P, c, s, us, ts, qst, a, b, d);
    us = a;
    ts = b;
    qst = d;
    tau = t1;
}

// One application of the fixed-point map F (iterate_interface_state) to the
// state x = (u*, theta*, q*[, T_s]); the surface constants s0 are copied.
template <class R, bool SKIN>
__device__ __forceinline__ void eval_map(const DevIface<R>& P, const CellConst<R>& c, const SurfaceConst<R>& s0,
                                         const R* x, R* y, bool* pinned = nullptr) {
    SurfaceConst<R> s = s0;
    R us = x[0], ts = x[1], qs = x[2];
    if (SKIN) s.Ts = x[3];
    iterate_state<R, SKIN>(P, c, s, us, ts, qs, pinned);
    y[0] = us; y[1] = ts; y[2] = qs;
    if (SKIN) y[3] = s.Ts;
}

// Inverse of the N x N matrix a (Gauss-Jordan, partial pivoting; a is destroyed).
// Returns false when a pivot vanishes.
template <int N>
__device__ __forceinline__ bool invert(float (&a)[N][N], float (&inv)[N][N]) {
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) inv[i][j] = i == j ? 1.0f : 0.0f;
#pragma unroll
    for (int k = 0; k < N; k++) {
        int piv = k;
        float best = fabsf(a[k][k]);
#pragma unroll
        for (int i = k + 1; i < N; i++)
            if (fabsf(a[i][k]) > best) { best = fabsf(a[i][k]); piv = i; }
        if (!(best > 0.0f)) return false;
        if (piv != k) {
#pragma unroll
            for (int j = 0; j < N; j++) {
                float t = a[k][j]; a[k][j] = a[piv][j]; a[piv][j] = t;
                t = inv[k][j]; inv[k][j] = inv[piv][j]; inv[piv][j] = t;
            }
        }
        float d = 1.0f / a[k][k];
#pragma unroll
        for (int j = 0; j < N; j++) { a[k][j] *= d; inv[k][j] *= d; }
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (i == k) continue;
            float m = a[i][k];
#pragma unroll
            for (int j = 0; j < N; j++) { a[i][j] -= m * a[k][j]; inv[i][j] -= m * inv[k][j]; }
        }
    }
    return true;
}

// The reference's FP64 fixed point from (us, ts, qst) and s64. Returns iterations.
template <bool SKIN, bool QSKIN = false, bool PAIR = false, class R = double>
__device__ __forceinline__ int solve_plain(const DevIface<R>& P64, const CellConst<R>& c64,
                                           SurfaceConst<R>& s64, R& us, R& ts, R& qst,
                                           bool& nonconv, LanePair lp = LanePair{0u, 0}) {
    R drift;
    int it = fixed_point<R, SKIN, QSKIN, PAIR>(P64, c64, s64, us, ts, qst, P64.maxiter, drift, lp);
    nonconv = P64.stop_kind == NESF_STOP_CONVERGENCE && !(drift < P64.tol);
    return it;
}

// Negligible magnitudes of u*, theta*, q*, T_s (relative errors below them are
// measured against these).
__device__ __forceinline__ float state_floor(int i) {
    return i == 0 ? 1e-4f : (i == 1 ? 1e-5f : (i == 2 ? 1e-8f : 1e-3f));
}

// Central-difference step of the Jacobian column of state component k: large
// enough that FP32 rounding of F (T_s carries only ~1.5e-5 K at 270 K) stays far
// below the difference, small enough that the O(h^2) curvature error is negligible.
__device__ __forceinline__ float jac_step(int k, float xk) {
    return k == 3 ? 0.05f : fmaxf(1e-2f * fabsf(xk), state_floor(k));
}

enum ReplayReason { REPLAY_CALM = 0, REPLAY_NO_FP32 = 1, REPLAY_SLOW = 2, REPLAY_BOUND = 3, REPLAY_SINGULAR = 4 };

// What solve_fast decided for a cell.
enum FastOutcome { FAST_SOLVED = 0, FAST_POLISH = 1, FAST_REPLAY = 2 };

// Infinity norm (max row sum) of an N x N matrix.
template <int N>
__device__ __forceinline__ float inf_norm(const float (&a)[N][N]) {
    float n = 0.0f;
#pragma unroll
    for (int i = 0; i < N; i++) {
        float r = 0.0f;
#pragma unroll
        for (int j = 0; j < N; j++) r += fabsf(a[i][j]);
        n = fmaxf(n, r);   // fmaxf drops a NaN row: the caller checks the sum below
    }
    return n;
}

// Upper bound of the spectral radius of J from Gelfand's formula on the 32nd
// power, ||J^32||^(1/32) >= rho(J) in any induced norm; J^32 comes from five
// squarings with the norm taken out at each. Unlike a power-iteration ratio it
// is not fooled by a complex pair of dominant eigenvalues (a damped rotation of
// the state, common with a skin temperature). +inf when J holds a NaN.
template <int N>
__device__ __forceinline__ float spectral_bound(const float (&J)[N][N]) {
    float A[N][N];
    float chk = 0.0f;
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) { A[i][j] = J[i][j]; chk += J[i][j]; }
    if (chk != chk) return M<float>::inf();
    float e = 0.0f;   // J^(2^s) = A * exp(e)
#pragma unroll 1
    for (int s = 0; s < 5; s++) {
        float n = inf_norm<N>(A);
        if (!(n > 0.0f)) return 0.0f;   // nilpotent at FP32 resolution
        e = 2.0f * (e + logf(n));
        float inv = 1.0f / n;
        float B[N][N];
#pragma unroll
        for (int i = 0; i < N; i++)
#pragma unroll
            for (int j = 0; j < N; j++) B[i][j] = A[i][j] * inv;
#pragma unroll
        for (int i = 0; i < N; i++)
#pragma unroll
            for (int j = 0; j < N; j++) {
                float t = 0.0f;
#pragma unroll
                for (int k = 0; k < N; k++) t += B[i][k] * B[k][j];
                A[i][j] = t;
            }
    }
    float n = inf_norm<N>(A);
    if (!(n > 0.0f)) return 0.0f;
    return expf((logf(n) + e) * (1.0f / 32.0f));
}

// The FP32 sweep of a cell over the FP32 inputs of the map (c32, s32; with a skin
// temperature the anchors `anc` and the state's fourth component tau = T_s -
// theta_a, the delta form), as a state machine that one map evaluation at a time
// advances (struct Sweep), so that a kernel can run the evaluations of cells that
// are at different stages of their sweeps in lockstep (the refill pass 1).
// sweep_fp32 runs one cell's machine to its end. x holds the start (u*, theta*,
// q*, tau) and, at the end, the FP32 fixed point. Outcomes: FAST_REPLAY (the cell
// must follow the reference's FP64 iteration; `reason` says why), FAST_SOLVED
// (ACCEPT32 only: the FP32 result is kept) or FAST_POLISH (the FP32 result needs
// FP64 Newton steps: J and rho_est are set for them). `fp32_it` counts FP32 map
// evaluations.
//
// ACCEPT32 (ADAPTIVE): the FP32 result is kept when F contracts by at most
// so.fp32_rho. STRICT (ADAPTIVE's passes): the sweep runs until every component,
// not just the drift sum, is converged at FP32 resolution -- the polish pass of
// the cells that pass 1 did not keep repeats pass 1's sweep exactly, so it reaches
// the same decisions.
//
// Bulk temperature (N = 3): J is a forward difference around the sweep's last
// evaluated point x_b (whose image y_b = F(x_b) the sweep already has), N map
// evaluations, enough for the decisions (rho, the replay rules, ADAPTIVE's
// acceptance), which tolerate its O(h) bias. CENTRAL (the cells that go on to FP64
// Newton steps): after the decisions the N mirrored points are evaluated too and J
// becomes the central difference, O(h^2), which the Newton steps' convergence needs
// on slowly contracting cells. Pass 1 of ADAPTIVE takes no CENTRAL: its polish
// pass repeats the sweep (same decisions) with CENTRAL. Skin temperature (N = 4):
// the central difference around x from the start, 2N evaluations (the forward
// scheme's extra state costs these kernels more in spills than it saves).
//
// The FP32 sweep and the Jacobian's evaluations run through one loop around a
// single inlined copy of the map, so a warp executes the same instructions for
// all of them: the kernel's hot code stays small enough for the instruction cache.
enum { SWEEP_CONTINUE = -1, SWEEP_DECIDE = -2 };

template <bool SKIN, bool ACCEPT32, bool STRICT = ACCEPT32, bool CENTRAL = !ACCEPT32>
struct Sweep {
    static constexpr int N = SKIN ? 4 : 3;
    static constexpr bool FWD = !SKIN;   // forward-difference J (bulk temperature)
    float x[4], x0[4];
    float yw[4];          // first iterate from the warm start while the cold start is probed
    float rw;
    float xb[4], yb[4];   // FWD: the last sweep point and its image, the Jacobian's base
    float yp[4];          // !FWD: F(x + h e_j) of the column in progress
    float J[N][N];
    SweepTrace tr;
    float prev, h, cond, rho_est;
    int probes, rising, it, phase, fp32_it, reason;
    // phase 0 sweep; 1 cold-start probe; FWD: 2 + j: F(x_b + h e_j), N + 2 + j: F(x_b - h e_j);
    // !FWD: 2 + 2j / 3 + 2j: F(x + h e_j) / F(x - h e_j)
    bool warm, decided, stalled, fell_back;   // decided (FWD): CENTRAL's mirrored points follow;
                                              // stalled: the sweep ended on the rising-drift rule

    // Start from x (the reference's start) or, with a warm start, the network's (u*, theta*,
    // q*) guess xw; T_s keeps its own.
    __device__ __forceinline__ void begin(const float (&start)[4], const float* xw) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            x[k] = x0[k] = start[k];
            yw[k] = xb[k] = yb[k] = yp[k] = 0.0f;
        }
        warm = xw != nullptr && isfinite(xw[0]) && isfinite(xw[1]) && isfinite(xw[2]) && xw[0] > 0.0f;
        if (warm) { x[0] = xw[0]; x[1] = xw[1]; x[2] = xw[2]; }
        rw = 0.0f;
        probes = 0;
        decided = stalled = fell_back = false;
        tr.d[0] = tr.d[1] = tr.d[2] = 0.0f;
        tr.lam = 1.0f;
        prev = M<float>::inf();
        rising = it = phase = fp32_it = 0;
        reason = -1;
        h = 0.0f;
        cond = 1.0f;      // condition of the anchored differences at the last sweep iterate
        rho_est = 0.0f;
    }

    // The point the map is evaluated at next.
    __device__ __forceinline__ void input(float (&xin)[4]) {
#pragma unroll
        for (int k = 0; k < 4; k++) xin[k] = phase == 1 ? x0[k] : x[k];
        if (phase >= 2) {
            const bool minus = FWD ? phase >= N + 2 : (phase & 1) != 0;
            const int jj = FWD ? phase - (minus ? N + 2 : 2) : (phase - 2) >> 1;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (FWD) xin[k] = xb[k];
                if (k == jj) { h = jac_step(k, xin[k]); xin[k] += minus ? -h : h; }
            }
        }
    }

    // Takes y = F(xin) (cd: the condition of the anchored differences of that evaluation).
    // Returns SWEEP_CONTINUE (evaluate the next input), SWEEP_DECIDE (the Jacobian is
    // complete: call decide) or an outcome.
    __device__ __forceinline__ int advance(const float (&xin)[4], const float (&y)[4], float cd,
                                           const DevIface<float>& P32, const SolveOpts& so) {
        const float tol = P32.tol;
        if (SKIN && phase == 0) cond = cd;
        if (phase == 1) {
            // cold-start fallback: keep the warm start unless its first residual, relative to
            // its state, exceeds fallback_ratio times the cold start's relative first residual
            probes = 1;
            float rc = fabsf(y[0] - x0[0]) + fabsf(y[1] - x0[1]) + fabsf(y[2] - x0[2]);
            float nw = fabsf(x[0]) + fabsf(x[1]) + fabsf(x[2]), nc = fabsf(x0[0]) + fabsf(x0[1]) + fabsf(x0[2]);
            const bool cold = !(rw * nc <= so.fallback_ratio * rc * nw);
            if (cold) fell_back = true;
            // from (cold ? x0 : x) to (cold ? y : yw), element by element (no pointer to a
            // member array, which would keep the whole state out of registers)
#pragma unroll
            for (int k = 0; k < 3; k++) tr.d[k] = fabsf((cold ? y[k] : yw[k]) - (cold ? x0[k] : x[k]));
            tr.lam = 1.0f;
            prev = cold ? rc : rw;
#pragma unroll
            for (int k = 0; k < 4; k++) x[k] = cold ? y[k] : yw[k];
            phase = 0;
            return SWEEP_CONTINUE;
        }
        if (phase == 0) {
            it++;
            float du = fabsf(y[0] - x[0]), dt = fabsf(y[1] - x[1]), dq = fabsf(y[2] - x[2]);
            float dT = SKIN ? fabsf(y[3] - x[3]) : 0.0f;
            float drift = du + dt + dq;
            if (warm && it == 1 && drift > 0.01f * (fabsf(x[0]) + fabsf(x[1]) + fabsf(x[2]))) {
                // a large first residual from the guess: probe the cold start before going on
#pragma unroll
                for (int k = 0; k < 4; k++) yw[k] = y[k];
                rw = drift;
                phase = 1;
                return SWEEP_CONTINUE;
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (FWD) { xb[k] = xin[k]; yb[k] = y[k]; }
                x[k] = y[k];
            }
            // FP32 resolution of the drift sum: the ulps of the scales themselves
            float res = 1.1920929e-7f * (fabsf(x[0]) + fabsf(x[1]) + fabsf(x[2]));
            if (drift > 64.0f * res || it <= 2) {
                tr.d[0] = du; tr.d[1] = dt; tr.d[2] = dq;
                tr.lam = it > 1 ? drift / prev : 1.0f;
            }
            // each component within 4 of its own ulps (ADAPTIVE), or the sum within 8
            const float u4 = 4.0f * 1.1920929e-7f;
            // (tau to 1e-7 K besides: dtheta = -tau)
            bool quiet = STRICT ? (du <= u4 * fabsf(x[0]) && dt <= u4 * fabsf(x[1]) && dq <= u4 * fabsf(x[2]) &&
                                     dT <= u4 * fabsf(x[3]) + 1e-7f)
                                  : drift <= 8.0f * res;
            bool done = drift < tol || quiet;
            if (!done && drift <= 1024.0f * res && drift >= prev) { done = ++rising >= 2; stalled = done; }
            else if (!done) rising = 0;
            prev = drift;
            if (done) {
                // calm cells: the reference's absolute drift rule leaves tol / u* of relative room
                if (fabsf(x[0]) * so.path_tol < tol) { fp32_it = it; reason = REPLAY_CALM; return FAST_REPLAY; }
                phase = 2;
            } else if (it >= P32.maxiter) {
                fp32_it = it;
                reason = REPLAY_NO_FP32;
                return FAST_REPLAY;                       // no FP32 convergence
            }
            return SWEEP_CONTINUE;
        }
        if (!FWD && !(phase & 1)) {
#pragma unroll
            for (int k = 0; k < 4; k++) yp[k] = y[k];
            phase++;
            return SWEEP_CONTINUE;
        }
        if (!FWD) {
            // central difference: column (phase - 3) / 2
            const int jj = (phase - 3) >> 1;
            const float inv2h = 0.5f / h;
#pragma unroll
            for (int ii = 0; ii < N; ii++)
#pragma unroll
                for (int k = 0; k < N; k++)
                    if (k == jj) J[ii][k] = (yp[ii] - y[ii]) * inv2h;
            return ++phase == 2 * N + 2 ? SWEEP_DECIDE : SWEEP_CONTINUE;
        }
        if (phase < N + 2) {
            // forward difference: column phase - 2
            const int jj = phase - 2;
            const float invh = 1.0f / h;
#pragma unroll
            for (int ii = 0; ii < N; ii++)
#pragma unroll
                for (int k = 0; k < N; k++)
                    if (k == jj) J[ii][k] = (y[ii] - yb[ii]) * invh;
            return ++phase == N + 2 ? SWEEP_DECIDE : SWEEP_CONTINUE;
        }
        // the mirrored point of column phase - N - 2: the forward column becomes the central
        // difference (F(x_b + h e_j) - F(x_b - h e_j)) / 2h, F(x_b + h e_j) = y_b + h J e_j
        const int jj = phase - (N + 2);
        const float inv2h = 0.5f / h;
#pragma unroll
        for (int ii = 0; ii < N; ii++)
#pragma unroll
            for (int k = 0; k < N; k++)
                if (k == jj) J[ii][k] = (J[ii][k] * h + yb[ii] - y[ii]) * inv2h;
        if (++phase < 2 * N + 2) return SWEEP_CONTINUE;
        // CENTRAL: the mirrored points are in J; the decisions were made before them
        fp32_it += N;
        return FAST_POLISH;
    }

    // The decisions once the Jacobian is complete: an outcome, or SWEEP_CONTINUE when
    // CENTRAL's mirrored points are to be evaluated first.
    __device__ __forceinline__ int decide(const SolveOpts& so, const DevIface<float>& P32) {
        const float tol = P32.tol;
        fp32_it = it + probes + (FWD ? N : 2 * N);
        // ---- contraction rate of F at the solution
        rho_est = spectral_bound<N>(J);
        if (!(rho_est < 0.995f)) { reason = REPLAY_SLOW; return FAST_REPLAY; }
        // ---- the reference's stopping error along its slowest mode: e = rho / (1 - rho) d, |d|_1 < tol.
        // Mode shape: power iteration from the last drift (each component's largest share over the
        // last two iterates, which a rotating complex mode alternates between), or the last drift.
        float v[4] = {tr.d[0], tr.d[1], tr.d[2], 0.0f};
        float vn = v[0] + v[1] + v[2];
        if (vn > 0.0f) {
            float frac[3] = {v[0] / vn, v[1] / vn, v[2] / vn};
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int ii = 0; ii < N; ii++)
#pragma unroll
                    for (int jj = 0; jj < N; jj++) w[ii] += J[ii][jj] * v[jj];
                float wn = 0.0f;
#pragma unroll
                for (int ii = 0; ii < N; ii++) wn += fabsf(w[ii]);
                if (!(wn > 0.0f)) break;          // J nilpotent on the drift: keep the drift's shape
                float inv = 1.0f / wn;
#pragma unroll
                for (int ii = 0; ii < N; ii++) v[ii] = w[ii] * inv;   // signed: J's modes, not |J|'s
                float mn = fabsf(v[0]) + fabsf(v[1]) + fabsf(v[2]);
                if (k >= 6 && mn > 0.0f) {
#pragma unroll
                    for (int ii = 0; ii < 3; ii++)
                        frac[ii] = k == 6 ? fabsf(v[ii]) / mn : fmaxf(frac[ii], fabsf(v[ii]) / mn);
                }
            }
            float kb = rho_est / (1.0f - rho_est) * tol;
#pragma unroll
            for (int ii = 0; ii < 3; ii++)
                if (!(kb * frac[ii] <= so.path_tol * fmaxf(fabsf(x[ii]), state_floor(ii)))) {
                    reason = REPLAY_BOUND;
                    return FAST_REPLAY;
                }
        }
        // ---- ADAPTIVE: keep the FP32 result of a quiet, well-contracting cell
        // FP32 rounding of the anchored terms (~1e-7 of each), amplified by their
        // cancellation and by 1 / (1 - rho), must stay within path_tol
        if (ACCEPT32 && !stalled && rho_est <= so.fp32_rho && cond * 1.2e-7f <= so.path_tol * (1.0f - rho_est))
            return FAST_SOLVED;
        if (FWD && CENTRAL) {   // back to the map for the mirrored points (one copy of the map)
            decided = true;
            return SWEEP_CONTINUE;
        }
        return FAST_POLISH;
    }
};

// One FP32 evaluation of the map at xin (the sweep's inputs); cd receives the
// condition number of the anchored differences (skin temperature; 1 otherwise).
template <bool SKIN>
__device__ __forceinline__ void sweep_map(const DevIface<float>& P32, const CellConst<float>& c32,
                                          const SurfaceConst<float>& s32, const SkinAnchor<float>& anc,
                                          const float (&xin)[4], float (&y)[4], float& cd) {
    float yu = xin[0], yt = xin[1], yq = xin[2], yT = xin[3];
    cd = 1.0f;
    if (SKIN) {
        iterate_skin_delta<float>(P32, c32, anc, yu, yt, yq, yT, &cd);
    } else {
        SurfaceConst<float> sv = s32;
        iterate_state<float, false>(P32, c32, sv, yu, yt, yq);
    }
    y[0] = yu; y[1] = yt; y[2] = yq; y[3] = SKIN ? yT : 0.0f;   // (a constant fourth component without a skin)
}

template <bool SKIN, bool ACCEPT32, bool STRICT = ACCEPT32, bool CENTRAL = !ACCEPT32>
__device__ __forceinline__ int sweep_fp32(const DevIface<float>& P32, const CellConst<float>& c32,
                                          const SurfaceConst<float>& s32, const SkinAnchor<float>& anc,
                                          float (&x)[4], const SolveOpts& so, int& fp32_it, int& reason,
                                          float (&J)[SKIN ? 4 : 3][SKIN ? 4 : 3], float& rho_est,
                                          const float* xw, bool* fell_back) {
    constexpr int N = SKIN ? 4 : 3;
    Sweep<SKIN, ACCEPT32, STRICT, CENTRAL> sw;
    sw.begin(x, xw);
    int out;
    // the decisions run after the evaluation loop, where the lanes of a warp that left it
    // at different iterations are together again (inside it each lane would take them
    // alone); CENTRAL's mirrored points go back into the loop
#pragma unroll 1
    for (;;) {
#pragma unroll 1
        for (;;) {
            float xin[4], y[4], cd;
            sw.input(xin);
            sweep_map<SKIN>(P32, c32, s32, anc, xin, y, cd);
            out = sw.advance(xin, y, cd, P32, so);
            if (out != SWEEP_CONTINUE) break;
        }
        if (out != SWEEP_DECIDE) break;
        out = sw.decide(so, P32);
        if (out != SWEEP_CONTINUE) break;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = sw.x[k];
#pragma unroll
    for (int ii = 0; ii < N; ii++)
#pragma unroll
        for (int jj = 0; jj < N; jj++) J[ii][jj] = sw.J[ii][jj];
    fp32_it = sw.fp32_it;
    if (sw.reason >= 0) reason = sw.reason;
    rho_est = sw.rho_est;
    if (fell_back && sw.fell_back) *fell_back = true;
    return out;
}

// FP64 Newton steps on x = F(x) from the FP32 fixed point x of sweep_fp32 (J and
// rho_est its Jacobian and contraction bound), with the reference's FP64 cell
// constants (c64, s64). On FAST_SOLVED the solution is in us, ts, qst and, with a
// skin temperature, s64.Ts (the interface temperature; the rest of s64 is not
// updated); FAST_REPLAY (I - J singular) leaves them untouched. `fp64_it` counts
// FP64 map evaluations. R: double, or df (the steps in double-float arithmetic).
template <bool SKIN, class R = double>
__device__ __forceinline__ int newton_fp64(const DevIface<R>& P64, const CellConst<R>& c64,
                                           SurfaceConst<R>& s64, const float (&x)[4],
                                           const float (&J)[SKIN ? 4 : 3][SKIN ? 4 : 3], float rho_est,
                                           const SolveOpts& so, R& us, R& ts, R& qst, int& fp64_it,
                                           int& reason) {
    constexpr int N = SKIN ? 4 : 3;
    fp64_it = 0;
    float A[N][N], Ainv[N][N];
#pragma unroll
    for (int ii = 0; ii < N; ii++)
#pragma unroll
        for (int jj = 0; jj < N; jj++) A[ii][jj] = (ii == jj ? 1.0f : 0.0f) - J[ii][jj];
    if (!invert<N>(A, Ainv)) { reason = REPLAY_SINGULAR; return FAST_REPLAY; }
    float A3i[3][3];
    if (SKIN) {
        float A3[3][3];
#pragma unroll
        for (int ii = 0; ii < 3; ii++)
#pragma unroll
            for (int jj = 0; jj < 3; jj++) A3[ii][jj] = (ii == jj ? 1.0f : 0.0f) - J[ii][jj];
        if (!invert<3>(A3, A3i)) { reason = REPLAY_SINGULAR; return FAST_REPLAY; }
    }
    R xd[4] = {R(x[0]), R(x[1]), R(x[2]), SKIN ? c64.tha + R(x[3]) : R(0.0)};
    // a Newton step with an approximate J shrinks the error by about |dJ| / (1 - rho):
    // slowly contracting cells take more steps, up to polish_steps
    const int want = 1 + (rho_est > 0.5f ? 1 : 0) + (rho_est > 0.8f ? 1 : 0);
    const int cap = so.polish_steps > 0 ? so.polish_steps : 3;
    const int steps = want < cap ? want : cap;
#pragma unroll 1
    for (int n = 0; n < steps; n++) {
        R y[4];
        bool pinned = false;
        eval_map<R, SKIN>(P64, c64, s64, xd, y, &pinned);
        fp64_it++;
        float r[4];
#pragma unroll
        for (int ii = 0; ii < N; ii++) r[ii] = (float)(y[ii] - xd[ii]);
        float dl[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (SKIN && pinned) {
            // T_s sits on the melting cap (or the unconsolidated-ice branch): it is
            // y[3] exactly, and the Newton step runs on the three flux scales alone
#pragma unroll
            for (int ii = 0; ii < 3; ii++)
#pragma unroll
                for (int jj = 0; jj < 3; jj++) dl[ii] += A3i[ii][jj] * r[jj];
        } else {
#pragma unroll
            for (int ii = 0; ii < N; ii++)
#pragma unroll
                for (int jj = 0; jj < N; jj++) dl[ii] += Ainv[ii][jj] * r[jj];
        }
#pragma unroll
        for (int ii = 0; ii < 3; ii++) xd[ii] += R(dl[ii]);
        if (SKIN) xd[3] = pinned ? y[3] : xd[3] + R(dl[3]);
    }
    us = xd[0]; ts = xd[1]; qst = xd[2];
    if (SKIN) s64.Ts = xd[3];   // the callers read the interface temperature alone
    return FAST_SOLVED;
}

// ------------------------------------------ adaptive pass 1: FP32 in and out
// The inputs of an adaptive pass-1 cell: the map's constants in FP32, built from
// the FP32 loads, with FP64 only where differences cancel -- theta_a - T_s and
// q_a - q_s(T_s) for a bulk interface temperature (the surface constants s), the
// anchors of the delta form for a skin temperature (anc) -- and the flux epilogue
// in FP32. A kept FP32 result carries FP32 rounding anyway; the few FP64
// operations left per cell replace the reference epilogue's FP64 divisions, square
// roots and pow, which at 1/64 of the FP32 rate cost as much as the sweep.
struct Fast32 {
    CellConst<float> c;
    SurfaceConst<float> s;    // bulk interface temperature
    SkinAnchor<float> anc;    // skin temperature
    double tha;               // theta_a (a skin state's T_s = theta_a + tau)
    double Ts0;               // the interface temperature before the iteration
};

// theta_a - T_a = g h / cp_m(q_a) (surface_atmosphere_temperature), ~0.1 K. In FP64 or
// double-float: its FP32 rounding (~1e-8 K) would be a large part of a near-neutral
// theta_a - T_s.
template <class A>
__device__ __forceinline__ A lift_temperature(const DevIface<A>& P, A qa) {
    return P.g * P.h / cp_m(P, qa);
}

// Surface constants of a bulk interface temperature Ts: q_s and the differences in A,
// FP64 or double-float (from the fields' own T_a and q_a: FP64 fields are not rounded
// first), the rest in FP32 from the rounded T_s and q_s.
template <class A>
__device__ __forceinline__ void fast_surface(const DevIface<A>& P, const DevIface<float>& Pf, A Ta, A qa, A pa,
                                             A lift, A Ts, SurfaceConst<float>& s) {
    A qs = surface_specific_humidity<A, true>(P, pa, Ts);
    s.Ts = (float)Ts;
    s.qs = (float)qs;
    s.dth = (float)((Ta - Ts) + lift);
    s.dq = (float)(qa - qs);
    float Tv = virtual_temperature(Pf, s.Ts, s.qs);
    float delta = Pf.eps - 1.0f;
    s.gTv = Pf.g / Tv;
    s.A1 = 1.0f + delta * s.qs;
    s.A2 = delta * Tv;
    s.nu_u = air_viscosity(Pf.rough[0], s.Ts);
    s.nu_t = air_viscosity(Pf.rough[1], s.Ts);
    s.nu_q = air_viscosity(Pf.rough[2], s.Ts);
}

// The cancelling differences of an adaptive pass-1 cell, computed once by the classify pass
// in double-float (48 bits on the FP32 pipes: FP64 issues one warp instruction per ~64
// cycles per SM sub-partition on this GPU) and stored per work-list slot, so that pass 1
// loads them instead of taking FP64 steps in its prologue: 16 floats, the surface constants
// of a bulk interface temperature (10) or the skin anchors (10), the velocity difference
// (2), theta_a and the starting interface temperature as double-float pairs (4).
constexpr int kAnchorFloats = 16;

__device__ __forceinline__ void anchor_store(float* buf, int64_t slot, const float (&v)[kAnchorFloats]) {
    float4* p = reinterpret_cast<float4*>(buf + slot * kAnchorFloats);
#pragma unroll
    for (int q = 0; q < kAnchorFloats / 4; q++) p[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

template <bool SKIN>
__device__ __forceinline__ void anchor_pack(const SurfaceConst<float>& s, const SkinAnchor<float>& a, float du,
                                            float dv, df tha, df Ts0, float (&v)[kAnchorFloats]) {
    if (SKIN) {
        v[0] = a.dTi; v[1] = a.dTb; v[2] = a.dTm; v[3] = a.pva; v[4] = a.qsa;
        v[5] = a.dqa; v[6] = a.Qa0; v[7] = a.Iupa; v[8] = a.gA; v[9] = a.gK;
    } else {
        v[0] = s.Ts; v[1] = s.qs; v[2] = s.dth; v[3] = s.dq; v[4] = s.gTv;
        v[5] = s.A1; v[6] = s.A2; v[7] = s.nu_u; v[8] = s.nu_t; v[9] = s.nu_q;
    }
    v[10] = du; v[11] = dv;
    v[12] = tha.hi; v[13] = tha.lo; v[14] = Ts0.hi; v[15] = Ts0.lo;
}

// Loads a slot's record into the pass-1 state (f.c's velocity difference, f.s or f.anc,
// f.tha, f.Ts0).
template <bool SKIN>
__device__ __forceinline__ void anchor_load(const float* buf, int64_t slot, Fast32& f) {
    const float4* p = reinterpret_cast<const float4*>(buf + slot * kAnchorFloats);
    const float4 q0 = p[0], q1 = p[1], q2 = p[2], q3 = p[3];
    if (SKIN) {
        SkinAnchor<float>& a = f.anc;
        a.dTi = q0.x; a.dTb = q0.y; a.dTm = q0.z; a.pva = q0.w; a.qsa = q1.x;
        a.dqa = q1.y; a.Qa0 = q1.z; a.Iupa = q1.w; a.gA = q2.x; a.gK = q2.y;
    } else {
        SurfaceConst<float>& s = f.s;
        s.Ts = q0.x; s.qs = q0.y; s.dth = q0.z; s.dq = q0.w; s.gTv = q1.x;
        s.A1 = q1.y; s.A2 = q1.z; s.nu_u = q1.w; s.nu_t = q2.x; s.nu_q = q2.y;
    }
    f.c.du = q2.z;
    f.c.dv = q2.w;
    f.tha = (double)q3.x + (double)q3.y;
    f.Ts0 = (double)q3.z + (double)q3.w;
}

// Momentum flux direction: (-u*^2 du / |dU|, -u*^2 dv / |dU|) in FP32, in FP64 where
// |dU|^2 would underflow.
__device__ __forceinline__ void stress_fast(float us, float du, float dv, float& tx, float& ty) {
    float dU = sqrtf(du * du + dv * dv);
    if (dU < 1e-18f && (du != 0.0f || dv != 0.0f)) {
        double d = sqrt((double)du * du + (double)dv * dv);
        tx = (float)(-((double)us * us) * du / d);
        ty = (float)(-((double)us * us) * dv / d);
        return;
    }
    tx = dU == 0.0f ? 0.0f : -(us * us) * du / dU;
    ty = dU == 0.0f ? 0.0f : -(us * us) * dv / dU;
}

// FP32 sweep + FP64 Newton polish from the reference's FP64 cell constants (c64,
// s64), the FP32 inputs rounded from them. Outputs as newton_fp64's; `fp32_it`
// counts FP32 map evaluations. STRICT: the sweep of sweep_fp32<.., STRICT>.
template <bool SKIN, bool STRICT = false>
__device__ __forceinline__ int solve_fast(const DevIface<double>& P64, const DevIface<float>& P32,
                                          const CellConst<double>& c64, SurfaceConst<double>& s64, double& us,
                                          double& ts, double& qst, const SolveOpts& so, int& fp32_it, int& fp64_it,
                                          int& reason, const float* xw = nullptr, bool* fell_back = nullptr) {
    constexpr int N = SKIN ? 4 : 3;
    fp64_it = 0;
    CellConst<float> c32;
    SurfaceConst<float> s32;
    convert_const(c64, c32);
    convert_surface(s64, s32);
    SkinAnchor<float> anc{};
    if (SKIN) anc = skin_anchor(P64, c64.tha, c64.Ti, c64.Si, c64.qa, c64.pa, c64.sw, c64.lw);
    float x[4] = {(float)us, (float)ts, (float)qst, SKIN ? (float)(s64.Ts - c64.tha) : 0.0f};
    float J[N][N];
    float rho_est;
    if (sweep_fp32<SKIN, false, STRICT>(P32, c32, s32, anc, x, so, fp32_it, reason, J, rho_est, xw, fell_back) ==
        FAST_REPLAY)
        return FAST_REPLAY;
    return newton_fp64<SKIN>(P64, c64, s64, x, J, rho_est, so, us, ts, qst, fp64_it, reason);
}

// Warp-aggregated append of `id` to one side of a member's work list; returns the
// slot it took (member * per_member + position), or -1.
__device__ __forceinline__ int64_t worklist_push(const WorkList& w, int member, bool active, bool stable,
                                                 uint32_t id) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
    int64_t slot = -1;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        bool want = active && (stable == (side == 1));
        unsigned ballot = __ballot_sync(mask, want);
        if (ballot == 0) continue;
        int leader = __ffs(ballot) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&w.count[2 * member + side], (unsigned)__popc(ballot));
        base = __shfl_sync(mask, base, leader);
        if (want) {
            unsigned pos = base + __popc(ballot & ((1u << lane) - 1u));
            int64_t p = side == 0 ? (int64_t)pos : w.per_member - 1 - (int64_t)pos;
            w.idx[(int64_t)member * w.per_member + p] = id;
            slot = (int64_t)member * w.per_member + p;
        }
    }
    return slot;
}

// The slot of the w-th entry of a member's work list (unstable cells first).
__device__ __forceinline__ int64_t worklist_slot(const WorkList& wl, int member, int64_t w) {
    const unsigned nu = wl.count[2 * member];
    return (int64_t)member * wl.per_member + (w < nu ? w : wl.per_member - 1 - (w - nu));
}

// The w-th entry of a member's work list (unstable cells first), or -1.
__device__ __forceinline__ int64_t worklist_get(const WorkList& wl, int member, int64_t w) {
    const unsigned nu = wl.count[2 * member], ns = wl.count[2 * member + 1];
    if (w >= (int64_t)nu + ns) return -1;
    const uint32_t* seg = wl.idx + (int64_t)member * wl.per_member;
    return w < nu ? (int64_t)seg[w] : (int64_t)seg[wl.per_member - 1 - (w - nu)];
}

// Sign class of the surface buoyancy flux from the interface state before the
// iteration (FP32): b* is proportional to dtheta (1 + delta q_s) + delta T_v dq
// (buoyancy_scale, similarity_theory_turbulent_fluxes.jl:417-425, with
// theta* = chi dtheta and q* = chi dq), so the cell's stability branch is fixed
// from the second iteration on.
__device__ __forceinline__ bool stable_class(const DevIface<float>& P, float Ta, float pa, float qa, float Ts) {
    float qs = surface_specific_humidity(P, pa, Ts);
    float tha = surface_atmosphere_temperature(P, Ta, qa);
    float dth = tha - Ts, dq = qa - qs;
    float delta = P.eps - 1.0f;
    float Tv = virtual_temperature(P, Ts, qs);
    return dth * (1.0f + delta * qs) + delta * Tv * dq > 0.0f;
}

// Warp-aggregated append of `id` to one part of the deferred-cell queue (lanes
// with want = true): part 0 the FP64 replays, part 1 the FP64 polishes.
// Warp-aggregated append of `id` to a queue part; returns its position there, or -1.
__device__ __forceinline__ int64_t queue_push(const ReplayQueue& q, int part, bool want, uint32_t id) {
    unsigned mask = __activemask();
    unsigned ballot = __ballot_sync(mask, want);
    if (!want) return -1;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&q.count[part], (unsigned)__popc(ballot));
    base = __shfl_sync(ballot, base, leader);
    unsigned pos = base + __popc(ballot & ((1u << lane) - 1u));
    if ((int64_t)pos >= q.capacity) return -1;
    q.idx[(int64_t)part * q.capacity + pos] = id;
    return (int64_t)pos;
}

__device__ __forceinline__ void replay_push(const ReplayQueue& q, bool want, uint32_t id, int part = 0) {
    queue_push(q, part, want, id);
}
__device__ __forceinline__ int64_t polish_push(const ReplayQueue& q, bool want, uint32_t id) {
    return queue_push(q, 1, want, id);
}

// The polish state of part-1 entry `pos` (kPolishStateFloats): x, J row by row, rho, the
// FP32 map evaluations.
template <int N>
__device__ __forceinline__ void polish_state_store(const ReplayQueue& q, int64_t pos, const float (&x)[4],
                                                   const float (&J)[N][N], float rho, int fp32_it) {
    float v[kPolishStateFloats];
#pragma unroll
    for (int k = 0; k < kPolishStateFloats; k++) v[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = x[k];
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) v[4 + 4 * i + j] = J[i][j];
    v[20] = rho;
    v[21] = __int_as_float(fp32_it);
    float4* p = reinterpret_cast<float4*>(q.pstate + pos * kPolishStateFloats);
#pragma unroll
    for (int k = 0; k < kPolishStateFloats / 4; k++) p[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
}

template <int N>
__device__ __forceinline__ void polish_state_load(const ReplayQueue& q, int64_t pos, float (&x)[4], float (&J)[N][N],
                                                  float& rho, int& fp32_it) {
    float v[kPolishStateFloats];
    const float4* p = reinterpret_cast<const float4*>(q.pstate + pos * kPolishStateFloats);
#pragma unroll
    for (int k = 0; k < kPolishStateFloats / 4; k++) {
        const float4 w = p[k];
        v[4 * k] = w.x; v[4 * k + 1] = w.y; v[4 * k + 2] = w.z; v[4 * k + 3] = w.w;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) x[k] = v[k];
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) J[i][j] = v[4 + 4 * i + j];
    rho = v[20];
    fp32_it = __float_as_int(v[21]);
}

// Pass 1 of the adaptive solver (one member, convergence stopping rule), every schedule in
// one loop: each lane holds a cell and advances its FP32 sweep one map evaluation per trip
// (Sweep), whatever stage -- sweep, cold-start probe, Jacobian column -- the cell is at, so
// the lanes of a warp evaluate the map in lockstep. The decisions, the epilogue (store or
// queue) and the taking of new cells happen at warp events only, together for the lanes
// concerned: an event comes when no lane is sweeping, or, with lane refill, when `refill`
// lanes are done or empty. Schedules:
//   fetch = false: so.cells work-list entries per thread (the grid covers the list once the
//     cells are counted: thread t takes entries t, t + T, ..., T the grid's threads), the next
//     one when all of the warp's cells are done, no refill;
//   fetch, refill = 32: the resident warps take the next entries (rq.count[kFetchCounter])
//     when all their cells are done -- warp fetching;
//   fetch, refill < 32: a warp takes new entries for its idle lanes as soon as `refill` of
//     them are idle -- lane refill: a cell that converges early frees its lane for a new
//     cell instead of holding it until the warp's slowest cell is done.
//   With fetching, each lane that needs entries reserves so.cells of them with the warp's one
//   atomic add (a warp of n such lanes advances the counter by n * cells; lane l of them owns
//   base + l, base + l + n, ...) and takes its reserved entries without another atomic.
// Every schedule runs the same instructions on a cell (one kernel, one inlined copy of the
// map), so the outputs do not depend on it. `Cell` is the interface's adapter: load(r,
// start) reads ring cell r's inputs into `f` and the start state, store(x, iterations)
// writes the fluxes of a kept FP32 result; `id` names the cell in the queues.
template <bool SKIN, class Cell>
__device__ __forceinline__ void adaptive_pass1(Cell& cell, const DevIface<float>& P32, const SolveOpts& so,
                                               const WorkList& wl, const ReplayQueue& rq, const float* guess,
                                               DevStats* stats, bool fetch) {
    const int lane = threadIdx.x & 31;
    const unsigned total = wl.count[0] + wl.count[1];
    const int refill = fetch ? (so.refill > 0 && so.refill < 32 ? so.refill : 32) : 32;
    const int cells = so.cells > 1 ? so.cells : 1;
    int taken = 0;                  // without fetching: entries this thread has taken
    unsigned rnext = 0, rstep = 0;  // with fetching: the lane's next reserved entry and its stride
    int rleft = 0;                  // and how many reserved entries are left
    Sweep<SKIN, true> sw;
    bool have = false, pending = false, alive = true;
    int outcome = SWEEP_CONTINUE;
#pragma unroll 1
    for (;;) {
        const unsigned running = __ballot_sync(0xffffffffu, have && !pending);
        const unsigned idle = __ballot_sync(0xffffffffu, pending || (!have && alive));
        if (running == 0u || (fetch && refill < 32 && __popc(idle) >= refill)) {
            if (pending) {   // the decisions and the epilogue of the lanes whose sweep is done
                if (outcome == SWEEP_DECIDE) outcome = sw.decide(so, P32);
                replay_push(rq, outcome == FAST_REPLAY, cell.id);
                const int64_t ps = polish_push(rq, outcome == FAST_POLISH, cell.id);
                if (SKIN && ps >= 0 && rq.pstate) polish_state_store(rq, ps, sw.x, sw.J, sw.rho_est, sw.fp32_it);
                if (outcome == FAST_SOLVED) {
                    cell.store(sw.x, sw.fp32_it);
                    if (stats) stats_add(stats, true, true, sw.fp32_it, false, false, 0, false, sw.fell_back);
                } else if (stats) {
                    stats_add(stats, true, false, 0, false, false, 0, outcome == FAST_REPLAY, sw.fell_back);
                    if (outcome == FAST_REPLAY) stats_replay_reason(stats, sw.reason);
                }
                have = pending = false;
            }
            int64_t w = -1;
            if (fetch) {
                const bool need = alive && !have;
                const unsigned nb = __ballot_sync(0xffffffffu, need && rleft == 0);
                if (nb) {
                    const int leader = __ffs(nb) - 1;
                    const unsigned n = (unsigned)__popc(nb);
                    unsigned base = 0;
                    if (lane == leader) base = atomicAdd(&rq.count[kFetchCounter], n * (unsigned)cells);
                    base = __shfl_sync(0xffffffffu, base, leader);
                    if (need && rleft == 0) {
                        rnext = base + (unsigned)__popc(nb & ((1u << lane) - 1u));
                        rstep = n;
                        rleft = cells;
                    }
                }
                if (need) {   // a reserved entry is at hand
                    const unsigned pos = rnext;
                    rnext += rstep;
                    rleft--;
                    if (pos < total) w = pos;
                    else {      // the later reserved entries lie beyond the list too
                        alive = false;
                        rleft = 0;
                    }
                }
            } else if (!have && taken < cells) {
                const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x +
                                  (int64_t)taken * gridDim.x * blockDim.x;
                taken++;
                if (t < (int64_t)total) w = t;
                if (w < 0 || taken == cells) alive = false;
            }
            if (w >= 0) {
                float xw[3], start[4];
                const int64_t slot = worklist_slot(wl, 0, w);
                const float* warm = mlp::guess_at(guess, slot, xw);
                cell.load(worklist_get(wl, 0, w), slot, start);
                sw.begin(start, warm);
                have = true;
            }
            if (!__any_sync(0xffffffffu, have)) break;
        }
        if (have && !pending) {
            float xin[4], y[4], cd;
            sw.input(xin);
            sweep_map<SKIN>(P32, cell.f.c, cell.f.s, cell.f.anc, xin, y, cd);
            outcome = sw.advance(xin, y, cd, P32, so);
            pending = outcome != SWEEP_CONTINUE;
        }
    }
}

// Grid of a pass-1 launch: with warp fetching, the blocks that can be resident at
// once (at most the one-thread-per-entry grid); otherwise that grid, divided by the
// cells each thread takes (adaptive pass 1).
template <class K>
inline dim3 pass1_grid(K kernel, dim3 grid, int threads, int sms, bool fetch, int cells = 1) {
    if (!fetch) {
        if (cells > 1) grid.x = (grid.x + (unsigned)cells - 1) / (unsigned)cells;
        return grid;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    const unsigned g = (unsigned)sms * (unsigned)per_sm;
    if (g < grid.x) grid.x = g;
    return grid;
}

// A host hook inside a solve's launch, for the coupling step's lanes. Atmosphere-ocean: after
// the classify pass and the inference, `ready` (optional) is recorded on the solve's stream,
// then fn(arg) runs. Atmosphere-sea-ice: after pass 1, fn(arg) runs, and the polish pass waits
// for `wait` (optional). fn enqueues work of another lane; a non-zero status from it is kept
// in `status` and ends the launch.
struct MidHook {
    int (*fn)(void*);
    void* arg;
    int status;
    cudaEvent_t ready;
    cudaEvent_t wait;
};

// before_pass1 (optional): an event the stream waits for after the classify pass and the
// warm-start inference, before pass 1. tail (optional): a second lane on which pass 1's
// replays run beside the polish pass (the queue's part 2 then holds the polish pass's).
// mid (optional): the hook above, run before the wait for before_pass1 is enqueued.
cudaError_t launch_ao(const AOArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t before_pass1 = nullptr, const TailLane* tail = nullptr,
                      MidHook* mid = nullptr);
cudaError_t launch_ao(const AOArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t before_pass1 = nullptr, const TailLane* tail = nullptr,
                      MidHook* mid = nullptr);
// Loads (under lazy module loading) every kernel that the one-member atmosphere-ocean
// solve of storage S can launch, so that a later launch loads no module.
cudaError_t preload_ao_kernels(const AOArgs<double>*);
cudaError_t preload_ao_kernels(const AOArgs<float>*);
// after_solve (optional): recorded once the pass-1 solve is enqueued.
// tail (optional): a second stream on which pass 1's replays run beside the polish pass.
// early (optional): a third stream on which the calm cells' replays run from the classify
// pass on, beside pass 1 (SolveOpts::calm_wind; without it no cell is sent early).
// before_pass1 (optional): an event the stream waits for before pass 1. mid (optional): the
// hook above, run after pass 1.
cudaError_t launch_ai(const AIArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t after_solve = nullptr, const TailLane* tail = nullptr,
                      const TailLane* early = nullptr, cudaEvent_t before_pass1 = nullptr, MidHook* mid = nullptr);
cudaError_t launch_ai(const AIArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, const WarmStart& ws, DevStats* stats,
                      cudaStream_t stream, cudaEvent_t after_solve = nullptr, const TailLane* tail = nullptr,
                      const TailLane* early = nullptr, cudaEvent_t before_pass1 = nullptr, MidHook* mid = nullptr);
cudaError_t launch_al(const ALArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, DevStats* stats, cudaStream_t stream);
cudaError_t launch_al(const ALArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, DevStats* stats, cudaStream_t stream);
template <class S>
cudaError_t launch_ao_samples(const AOArgs<S>& a, const DevIface<float>& P32, float* feat, float* targ,
                              cudaStream_t s);
// The adaptive solvers' replays in double-float arithmetic (one member), compiled apart
// (NESF_DF_PART 1 of the solve files).
cudaError_t launch_ai_replay_df(const AIArgs<double>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                DevStats* stats, unsigned grid, cudaStream_t s);
cudaError_t launch_ai_replay_df(const AIArgs<float>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                DevStats* stats, unsigned grid, cudaStream_t s);
cudaError_t launch_ao_replay_df(const AOArgs<double>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                bool skin, DevStats* stats, unsigned grid, cudaStream_t s);
cudaError_t launch_ao_replay_df(const AOArgs<float>& a, const DevIface<df>& P, const ReplayQueue& rq, int part,
                                bool skin, DevStats* stats, unsigned grid, cudaStream_t s);
cudaError_t preload_ao_replay_df(const AOArgs<double>*);
cudaError_t preload_ao_replay_df(const AOArgs<float>*);
// A solve's parameters in the arithmetic R of its deferred passes: member m's FP64 ones for an
// ensemble (ps), else p.
template <class R>
__device__ __forceinline__ const DevIface<R>& member_params(const DevIface<R>& p, const DevIface<double>* ps,
                                                            int64_t m) {
    if constexpr (std::is_same<R, double>::value) return ps ? ps[m] : p;
    else return p;
}
// The warm-start network's inference pass over a work list (nesf_mlp.cu).
cudaError_t mlp_pass(void* blob, const float* x, const float* t, float* y, int64_t n, const unsigned int* count,
                     int64_t per_member, int grid, bool state, cudaStream_t s);

}  // namespace nesf
