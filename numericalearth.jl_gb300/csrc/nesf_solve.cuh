// nesf_solve.cuh -- kernel argument bundles and launchers of the similarity-theory solves.
#pragma once

#include "nesf_kernels.cuh"

namespace nesf {

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
// Runs the FP32 fixed point. Returns the number of FP32 iterations and sets
// `state`: 0 converged (drift < tol), 1 stalled at FP32 resolution, 2 maxiter.
template <bool SKIN>
__device__ __forceinline__ int f32_sweep(const DevIface<float>& P, const CellConst<float>& c, SurfaceConst<float>& s,
                                         float& us, float& ts, float& qst, int maxiter, int& state) {
    int it = 0;
    float prev = M<float>::inf();
    int rising = 0;
    state = 2;
    while (it < maxiter) {
        float u0 = us, t0 = ts, q0 = qst;
        iterate_state<float, SKIN>(P, c, s, us, ts, qst);
        it++;
        float drift = fabsf(us - u0) + fabsf(ts - t0) + fabsf(qst - q0);
        if (drift < P.tol) { state = 0; break; }
        // FP32 resolution of the drift sum: a few ulps of the scales themselves
        float res = 8.0f * 1.1920929e-7f * (fabsf(us) + fabsf(ts) + fabsf(qst));
        if (drift <= res) { state = 1; break; }
        if (drift >= prev) {
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

// Solve one cell from the cold start u* = theta* = q* = 1e-4 (or a warm start).
// Returns iterations (FP32 + FP64); fills polish info.
template <int PREC, bool SKIN>
__device__ __forceinline__ int solve_cell(const DevIface<double>& P64, const DevIface<float>& P32,
                                          const CellConst<double>& c64, SurfaceConst<double>& s64, double& us,
                                          double& ts, double& qst, int polish_maxiter, bool& nonconv, int& piters) {
    piters = 0;
    if (PREC == NESF_PLAIN_F64 || P64.stop_kind == NESF_STOP_FIXED_ITERATIONS) {
        double drift;
        int it = fixed_point<double, SKIN>(P64, c64, s64, us, ts, qst, P64.maxiter, drift);
        nonconv = P64.stop_kind == NESF_STOP_CONVERGENCE && !(drift < P64.tol);
        return it;
    }
    CellConst<float> c32;
    SurfaceConst<float> s32;
    convert_const(c64, c32);
    convert_surface(s64, s32);
    float u = (float)us, t = (float)ts, q = (float)qst;
    int state;
    int it = f32_sweep<SKIN>(P32, c32, s32, u, t, q, P32.maxiter, state);
    us = u; ts = t; qst = q;
    nonconv = false;
    if (state != 0) {
        if (SKIN) {
            // continue the polish from the FP32 interface temperature
            s64.Ts = (double)s32.Ts;
        }
        double drift;
        piters = fixed_point<double, SKIN>(P64, c64, s64, us, ts, qst, polish_maxiter, drift);
        nonconv = state == 2 && !(drift < P64.tol);
    } else if (SKIN) {
        s64.Ts = (double)s32.Ts;
    }
    return it + piters;
}


cudaError_t launch_ao(const AOArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      int polish_maxiter, DevStats* stats, int block, cudaStream_t stream);
cudaError_t launch_ao(const AOArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      int polish_maxiter, DevStats* stats, int block, cudaStream_t stream);
cudaError_t launch_ai(const AIArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      int polish_maxiter, DevStats* stats, cudaStream_t stream);
cudaError_t launch_ai(const AIArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      int polish_maxiter, DevStats* stats, cudaStream_t stream);

}  // namespace nesf
