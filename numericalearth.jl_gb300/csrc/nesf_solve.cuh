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
#pragma once

#include "nesf_kernels.cuh"

namespace nesf {

// Knobs of the FP32 + FP64-polish solver.
struct SolveOpts {
    int polish_steps;   // FP64 Newton steps
    float path_tol;     // replay threshold on the reference's stopping-error bound
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

// Cells whose FP64 replay is deferred to the second pass.
struct ReplayQueue {
    uint32_t* idx;          // linear cell ids (member * ring + ring index)
    unsigned int* count;    // number of queued cells (zeroed before the first pass)
    int64_t capacity;
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

// Runs the FP32 fixed point from the reference's start. Returns the number of
// FP32 iterations and sets `state`: 0 converged (drift < tol), 1 stalled at FP32
// resolution, 2 reached maxiter.
template <bool SKIN>
__device__ __forceinline__ int f32_sweep(const DevIface<float>& P, const CellConst<float>& c, SurfaceConst<float>& s,
                                         float& us, float& ts, float& qst, int maxiter, int& state, SweepTrace& tr) {
    int it = 0;
    float prev = M<float>::inf();
    int rising = 0;
    state = 2;
    tr.d[0] = tr.d[1] = tr.d[2] = 0.0f;
    tr.lam = 1.0f;
    while (it < maxiter) {
        float u0 = us, t0 = ts, q0 = qst;
        iterate_state<float, SKIN>(P, c, s, us, ts, qst);
        it++;
        float du = fabsf(us - u0), dt = fabsf(ts - t0), dq = fabsf(qst - q0);
        float drift = du + dt + dq;
        // FP32 resolution of the drift sum: the ulps of the scales themselves
        float res = 1.1920929e-7f * (fabsf(us) + fabsf(ts) + fabsf(qst));
        if (drift > 64.0f * res || it <= 2) {
            tr.d[0] = du; tr.d[1] = dt; tr.d[2] = dq;
            tr.lam = it > 1 ? drift / prev : 1.0f;
        }
        if (drift < P.tol) { state = 0; break; }
        if (drift <= 8.0f * res) { state = 1; break; }
        if (drift <= 1024.0f * res && drift >= prev) {
            if (++rising >= 2) { state = 1; break; }
        } else {
            rising = 0;
        }
        prev = drift;
    }
    return it;
}

template <class R, class Q>
__device__ __forceinline__ void convert_const(const CellConst<R>& a, CellConst<Q>& b) {
    b.ua = Q(a.ua); b.va = Q(a.va); b.Ta = Q(a.Ta); b.pa = Q(a.pa); b.qa = Q(a.qa);
    b.ui = Q(a.ui); b.vi = Q(a.vi); b.Ti = Q(a.Ti); b.Si = Q(a.Si);
    b.hi = Q(a.hi); b.hs = Q(a.hs); b.hc = Q(a.hc); b.sw = Q(a.sw); b.lw = Q(a.lw); b.kappa = Q(a.kappa);
    b.du = Q(a.du); b.dv = Q(a.dv); b.dU2 = Q(a.dU2); b.tha = Q(a.tha);
    b.rho_a = Q(a.rho_a); b.cp_a = Q(a.cp_a); b.L_s = Q(a.L_s);
}

template <class R, class Q>
__device__ __forceinline__ void convert_surface(const SurfaceConst<R>& a, SurfaceConst<Q>& b) {
    b.Ts = Q(a.Ts); b.qs = Q(a.qs); b.dth = Q(a.dth); b.dq = Q(a.dq);
    b.gTv = Q(a.gTv); b.A1 = Q(a.A1); b.A2 = Q(a.A2);
    b.nu_u = Q(a.nu_u); b.nu_t = Q(a.nu_t); b.nu_q = Q(a.nu_q);
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
template <bool SKIN>
__device__ __forceinline__ int solve_plain(const DevIface<double>& P64, const CellConst<double>& c64,
                                           SurfaceConst<double>& s64, double& us, double& ts, double& qst,
                                           bool& nonconv) {
    double drift;
    int it = fixed_point<double, SKIN>(P64, c64, s64, us, ts, qst, P64.maxiter, drift);
    nonconv = P64.stop_kind == NESF_STOP_CONVERGENCE && !(drift < P64.tol);
    return it;
}

// Negligible magnitudes of u*, theta*, q*, T_s (relative errors below them are
// measured against these).
__device__ __forceinline__ float state_floor(int i) {
    return i == 0 ? 1e-4f : (i == 1 ? 1e-5f : (i == 2 ? 1e-8f : 1e-3f));
}

// FP32 sweep + FP64 Newton polish. Returns false when the cell must replay the
// reference's FP64 iteration (us, ts, qst, s64 are then untouched). On success
// the solution is in us, ts, qst and s64 (interface temperature); `fp32_it`
// counts FP32 map evaluations and `fp64_it` FP64 ones.
//
// The FP32 sweep and the N + 1 evaluations of the finite-difference Jacobian run
// through one loop around a single inlined copy of the map, so a warp executes
// the same instructions for both: the kernel's hot code stays small enough for
// the instruction cache.
// Central-difference step of the Jacobian column of state component k: large
// enough that FP32 rounding of F (T_s carries only ~1.5e-5 K at 270 K) stays far
// below the difference, small enough that the O(h^2) curvature error is negligible.
__device__ __forceinline__ float jac_step(int k, float xk) {
    return k == 3 ? 0.05f : fmaxf(1e-2f * fabsf(xk), state_floor(k));
}

enum ReplayReason { REPLAY_CALM = 0, REPLAY_NO_FP32 = 1, REPLAY_SLOW = 2, REPLAY_BOUND = 3, REPLAY_SINGULAR = 4 };

template <bool SKIN>
__device__ __forceinline__ bool solve_fast(const DevIface<double>& P64, const DevIface<float>& P32,
                                           const CellConst<double>& c64, SurfaceConst<double>& s64, double& us,
                                           double& ts, double& qst, const SolveOpts& so, int& fp32_it,
                                           int& fp64_it, int& reason) {
    constexpr int N = SKIN ? 4 : 3;
    fp64_it = 0;
    CellConst<float> c32;
    SurfaceConst<float> s32;
    convert_const(c64, c32);
    convert_surface(s64, s32);
    const float tol = (float)P64.tol;
    float x[4] = {(float)us, (float)ts, (float)qst, SKIN ? s32.Ts : 0.0f};   // sweep state
    float yp[4] = {0, 0, 0, 0};   // F(x + h e_j) of the column in progress
    float J[N][N];
    SweepTrace tr;
    tr.d[0] = tr.d[1] = tr.d[2] = 0.0f;
    tr.lam = 1.0f;
    float prev = M<float>::inf();
    int rising = 0;
    int it = 0;            // sweep iterations
    int phase = 0;         // 0 sweep; 2 + 2j / 3 + 2j: F(x + h e_j) / F(x - h e_j)
    float h = 0.0f;
    const int limit = P32.maxiter;
#pragma unroll 1
    for (;;) {
        float xin[4] = {x[0], x[1], x[2], x[3]};
        if (phase >= 2) {
            const int jj = (phase - 2) >> 1;
            const float sgn = (phase & 1) ? -1.0f : 1.0f;
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (k == jj) { h = jac_step(k, x[k]); xin[k] += sgn * h; }
        }
        SurfaceConst<float> sv = s32;
        if (SKIN) sv.Ts = xin[3];
        float yu = xin[0], yt = xin[1], yq = xin[2];
        iterate_state<float, SKIN>(P32, c32, sv, yu, yt, yq);
        float y[4] = {yu, yt, yq, SKIN ? sv.Ts : 0.0f};
        if (phase == 0) {
            it++;
            float du = fabsf(y[0] - x[0]), dt = fabsf(y[1] - x[1]), dq = fabsf(y[2] - x[2]);
            float drift = du + dt + dq;
#pragma unroll
            for (int k = 0; k < 4; k++) x[k] = y[k];
            // FP32 resolution of the drift sum: the ulps of the scales themselves
            float res = 1.1920929e-7f * (fabsf(x[0]) + fabsf(x[1]) + fabsf(x[2]));
            if (drift > 64.0f * res || it <= 2) {
                tr.d[0] = du; tr.d[1] = dt; tr.d[2] = dq;
                tr.lam = it > 1 ? drift / prev : 1.0f;
            }
            bool done = drift < tol || drift <= 8.0f * res;
            if (!done && drift <= 1024.0f * res && drift >= prev) done = ++rising >= 2;
            else if (!done) rising = 0;
            prev = drift;
            if (done) {
                // calm cells: the reference's absolute drift rule leaves tol / u* of relative room
                if (fabsf(x[0]) * so.path_tol < tol) { fp32_it = it; reason = REPLAY_CALM; return false; }
                phase = 2;
            } else if (it >= limit) {
                fp32_it = it;
                reason = REPLAY_NO_FP32;
                return false;                             // no FP32 convergence
            }
        } else if (!(phase & 1)) {
#pragma unroll
            for (int k = 0; k < 4; k++) yp[k] = y[k];
            phase++;
        } else {
            // central difference: column (phase - 3) / 2
            const int jj = (phase - 3) >> 1;
            const float inv2h = 0.5f / h;
#pragma unroll
            for (int ii = 0; ii < N; ii++)
#pragma unroll
                for (int k = 0; k < N; k++)
                    if (k == jj) J[ii][k] = (yp[ii] - y[ii]) * inv2h;
            if (++phase == 2 * N + 2) break;
        }
    }
    fp32_it = it + 2 * N;
    // ---- spectral radius and dominant mode of J (power iteration from the last drift)
    float v[4] = {tr.d[0], tr.d[1], tr.d[2], 0.0f};
    float vn = v[0] + v[1] + v[2];
    float rho_est = 0.0f;
    if (vn > 0.0f) {
        float rho = tr.lam, r2 = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int ii = 0; ii < N; ii++)
#pragma unroll
                for (int jj = 0; jj < N; jj++) w[ii] += J[ii][jj] * v[jj];
            float wn = 0.0f, vs = 0.0f;
#pragma unroll
            for (int ii = 0; ii < N; ii++) { wn += fabsf(w[ii]); vs += fabsf(v[ii]); }
            float g = vs > 0.0f ? wn / vs : 0.0f;
            if (k >= 6) r2 = k == 6 ? g : sqrtf(r2 * g);   // geometric mean of the last two ratios
            float inv = wn > 0.0f ? 1.0f / wn : 0.0f;
#pragma unroll
            for (int ii = 0; ii < N; ii++) v[ii] = w[ii] * inv;   // signed: the spectral radius of J, not of |J|
        }
        rho = r2 > 0.0f ? r2 : rho;
        rho_est = rho;
        // ---- the reference's stopping error along the mode: e = rho / (1 - rho) d, |d|_1 < tol
        if (!(rho < 0.995f)) { reason = REPLAY_SLOW; return false; }
        // mode shape: the power iteration's vector, or the last drift when J is nilpotent
        float mn = fabsf(v[0]) + fabsf(v[1]) + fabsf(v[2]);
        float k = rho / (1.0f - rho) * tol;
#pragma unroll
        for (int ii = 0; ii < 3; ii++) {
            float frac = r2 > 0.0f && mn > 0.0f ? fabsf(v[ii]) / mn : tr.d[ii] / vn;
            if (!(k * frac <= so.path_tol * fmaxf(fabsf(x[ii]), state_floor(ii)))) { reason = REPLAY_BOUND; return false; }
        }
    }
    // ---- FP64 Newton steps on x = F(x)
    float A[N][N], Ainv[N][N];
#pragma unroll
    for (int ii = 0; ii < N; ii++)
#pragma unroll
        for (int jj = 0; jj < N; jj++) A[ii][jj] = (ii == jj ? 1.0f : 0.0f) - J[ii][jj];
    if (!invert<N>(A, Ainv)) { reason = REPLAY_SINGULAR; return false; }
    float A3i[3][3];
    if (SKIN) {
        float A3[3][3];
#pragma unroll
        for (int ii = 0; ii < 3; ii++)
#pragma unroll
            for (int jj = 0; jj < 3; jj++) A3[ii][jj] = (ii == jj ? 1.0f : 0.0f) - J[ii][jj];
        if (!invert<3>(A3, A3i)) { reason = REPLAY_SINGULAR; return false; }
    }
    double xd[4] = {(double)x[0], (double)x[1], (double)x[2], SKIN ? (double)x[3] : 0.0};
    // a Newton step with an approximate J shrinks the error by about |dJ| / (1 - rho):
    // slowly contracting cells take more steps, up to polish_steps
    const int want = 1 + (rho_est > 0.5f ? 1 : 0) + (rho_est > 0.8f ? 1 : 0);
    const int cap = so.polish_steps > 0 ? so.polish_steps : 3;
    const int steps = want < cap ? want : cap;
#pragma unroll 1
    for (int n = 0; n < steps; n++) {
        double y[4];
        bool pinned = false;
        eval_map<double, SKIN>(P64, c64, s64, xd, y, &pinned);
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
        for (int ii = 0; ii < 3; ii++) xd[ii] += (double)dl[ii];
        if (SKIN) xd[3] = pinned ? y[3] : xd[3] + (double)dl[3];
    }
    us = xd[0]; ts = xd[1]; qst = xd[2];
    if (SKIN) {
        // the interface state that goes with the polished temperature
        s64.Ts = xd[3];
        double qs = surface_specific_humidity(P64, c64.pa, s64.Ts);
        surface_const(P64, c64, s64.Ts, qs, s64);
    }
    return true;
}

// Warp-aggregated append of `id` to one side of a member's work list.
__device__ __forceinline__ void worklist_push(const WorkList& w, int member, bool active, bool stable, uint32_t id) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
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
            uint32_t* seg = w.idx + (int64_t)member * w.per_member;
            if (side == 0) seg[pos] = id;
            else seg[w.per_member - 1 - pos] = id;
        }
    }
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

// Warp-aggregated append of `id` to the replay queue (lanes with want = true).
__device__ __forceinline__ void replay_push(const ReplayQueue& q, bool want, uint32_t id) {
    unsigned mask = __activemask();
    unsigned ballot = __ballot_sync(mask, want);
    if (!want) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(ballot) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(q.count, (unsigned)__popc(ballot));
    base = __shfl_sync(ballot, base, leader);
    unsigned pos = base + __popc(ballot & ((1u << lane) - 1u));
    if ((int64_t)pos < q.capacity) q.idx[pos] = id;
}

cudaError_t launch_ao(const AOArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, DevStats* stats, cudaStream_t stream);
cudaError_t launch_ao(const AOArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, DevStats* stats, cudaStream_t stream);
cudaError_t launch_ai(const AIArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, DevStats* stats, cudaStream_t stream);
cudaError_t launch_ai(const AIArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, const WorkList& wl, const ReplayQueue& rq, DevStats* stats, cudaStream_t stream);

}  // namespace nesf
