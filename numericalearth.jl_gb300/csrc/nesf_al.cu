// nesf_al.cu -- atmosphere-land similarity-theory (or coefficient-based) solve.
//
// _compute_atmosphere_land_interface_state! (InterfaceComputations/atmosphere_land_fluxes.jl:146-251)
//
// One thread per interior cell (the reference launches :xy), SoA loads of the
// exchange-grid atmosphere state and the land state (bulk temperature in
// kelvin, surface saturation). The surface does not move (u_s = v_s = 0), T_s is
// the bulk land temperature (BulkTemperature) and q_s follows the interface's
// land humidity model. PLAIN runs the reference's FP64 fixed point; the FP32
// modes run the FP32 sweep + FP64 Newton polish and replay, in place, the cells
// whose reference answer is path-dependent. SkinHumidity and DryLayerHumidity, whose
// q_s is iterated with the fluxes, always take the FP64 iteration.
#include <cfloat>

#include "nesf_solve.cuh"

namespace nesf {

// theta^(10/3) correctly rounded (the Millington-Quirk power, dry_layer_humidity.jl:262). The
// exponent is 10/3 rounded to double, p = 10/3 + d with d = 2^-51 / 3, so x^p = x^3 cbrt(x) x^d:
// x^3 as an exact double-double (fma products), cbrt(x) refined to double-double by one Newton
// step on c^3 = x, x^d = 1 + d ln x, and one rounding at the end. Where the vapor balance
// cancels, the fixed point amplifies a last-place change of this power a thousandfold, so the
// power must be the correctly rounded one that the reference's pow approximates.
__device__ __forceinline__ double pow_ten_thirds(double x) {
    if (!(x > 0x1p-300) || !(x < 0x1p300)) return pow(x, 10.0 / 3.0);
    const double x2 = x * x, x2l = fma(x, x, -x2);
    const double x3 = x2 * x, x3l = fma(x2, x, -x3) + x2l * x;
    const double c = cbrt(x);
    const double c2 = c * c, c2l = fma(c, c, -c2);
    const double c3 = c2 * c, c3l = fma(c2, c, -c3) + c2l * c;
    const double cl = -((c3 - x) + c3l) / (3.0 * c2);
    const double ph = x3 * c;
    double pl = fma(x3, c, -ph) + (x3 * cl + x3l * c);
    pl += ph * ((0x1p-51 / 3.0) * log(x));
    return ph + pl;
}

// DryLayerHumidity's per-cell constants (dry_layer_humidity.jl:317-365). The interface
// temperature is the bulk land temperature, so the front temperature
// T_e = T_in + chi (T_la - T_in) is T_la whatever chi = clamp(delta / l_T, 0, 1) is, and the
// front's source humidity and the saturated skin are both q_sat(T_la) = c.qres. What is left
// per cell is the dry layer's depth delta(S) (StorageBasedDryLayerDepth, :95-100), its
// conductance G_e = rho D_eff / max(delta, delta_min) (:252-263, 341-345) and the logistic
// weight of the series solution (:358-364).
__device__ __forceinline__ void dry_layer_constants(const DevIface<double>& P, double S, CellConst<double>& c) {
    using Md = M<double>;
    const double s = Md::fmin(S / P.dl_Sc, 1.0);
    const double delta = P.dl_max * pow(Md::fmax(1.0 - s, 0.0), P.dl_eta);
    double Dv = P.dl_D0;                                            // ConstantTortuosity
    if (P.tort == NESF_TORTUOSITY_POWER_LAW) {                      // Millington-Quirk
        const double theta_g = Md::fmax(P.dl_nu - Md::mul(S, P.dl_nu), 0.0);
        Dv = P.dl_D0 * pow_ten_thirds(theta_g) / (P.dl_nu * P.dl_nu);
    }
    c.Gq = c.rho_a * Dv / Md::fmax(delta, P.dl_min);
    const double z = 10.0 * Md::add(delta - P.dl_min, -(P.dl_w * 0.5)) / Md::fmax(P.dl_w, DBL_EPSILON);
    c.sig = 1.0 / (1.0 + exp(-z));
}

template <class S>
__device__ __forceinline__ void al_load(const DevIface<double>& P, const ALArgs<S>& a, int64_t k,
                                        CellConst<double>& c, double& qs) {
    c.ua = ld(a.ua, k); c.va = ld(a.va, k); c.Ta = ld(a.Ta, k); c.pa = ld(a.pa, k); c.qa = ld(a.qa, k);
    c.ui = c.vi = 0;                      // surface velocities are zero for land (:187-189)
    c.du = c.ua; c.dv = c.va;
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.Ti = ld(a.T, k);                    // bulk land temperature: the T_s of BulkTemperature (:173)
    c.Si = 0;
    c.hi = c.hs = c.hc = 0;
    c.sw = c.lw = 0;
    c.kappa = -1;
    c.Rth = 0;
    c.tha = surface_atmosphere_temperature(P, c.Ta, c.qa);
    c.rho_a = air_density(P, c.Ta, c.pa, c.qa);
    c.cp_a = c.L_s = 0;
    c.qres = surface_specific_humidity(P, c.pa, c.Ti);   // saturated at the bulk land temperature
    const double sat = a.sat ? ld(a.sat, k) : 1.0;
    c.Gq = P.skin_g;
    c.sig = 1.0;
    if (P.hum_form == NESF_HUMIDITY_DRY_LAYER) dry_layer_constants(P, sat, c);
    // the initial q_s is the saturation humidity (:200-201); BULK and FRACTIONAL recompute
    // it from the land state every iteration (a constant at a fixed T_s), SKIN and DRY_LAYER
    // iterate it
    qs = P.hum_form == NESF_HUMIDITY_SKIN || P.hum_form == NESF_HUMIDITY_DRY_LAYER ||
                 P.hum_form == NESF_HUMIDITY_IMPURE_SATURATION
             ? c.qres
             : land_humidity(P, c.pa, c.Ti, sat);
}

// The flux epilogue (atmosphere_land_fluxes.jl:216-250).
template <class S>
__device__ __forceinline__ void al_store(const DevIface<double>& P, const ALArgs<S>& a, int64_t k,
                                         const CellConst<double>& c, double us, double ts, double qst, double Ts,
                                         int iters) {
    double dU = sqrt(c.du * c.du + c.dv * c.dv);
    double tx = dU == 0 ? 0.0 : -(us * us) * c.du / dU;
    double ty = dU == 0 ? 0.0 : -(us * us) * c.dv / dU;
    double rho = c.rho_a;
    double cp = cp_m(P, c.qa);
    double Lv = latent_heat_vapor(P, c.Ta);
    st(a.Qv, k, -rho * Lv * us * qst);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    st(a.Ts, k, Ts);
    st(a.us, k, us);
    st(a.ts, k, ts);
    st(a.qs, k, qst);
    if (a.iters) a.iters[k] = iters;
}

template <class S, int PREC>
__global__ void __launch_bounds__(128) al_kernel(ALArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                 SolveOpts so, DevStats* stats) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    const int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    const int64_t k = a.L.at(i, j);
    const DevIface<double>& P = P64;
    CellConst<double> c;
    double qs0;
    al_load(P, a, k, c, qs0);
    SurfaceConst<double> s;
    surface_const(P, c, c.Ti, qs0, s);
    double us = 1e-4, ts = 1e-4, qst = 1e-4;   // :200-203
    int iters = 0, f64it = 0;
    bool nonconv = false, replayed = false;
    const bool needs = P.stop_kind == NESF_STOP_CONVERGENCE;
    if (P.hum_form == NESF_HUMIDITY_SKIN || P.hum_form == NESF_HUMIDITY_DRY_LAYER) {
        iters = solve_plain<false, true>(P, c, s, us, ts, qst, nonconv);
    } else if (PREC == NESF_PLAIN_F64 || !needs) {
        iters = solve_plain<false>(P, c, s, us, ts, qst, nonconv);
    } else {
        int f32it = 0, reason = -1;
        int outcome = solve_fast<false>(P, P32, c, s, us, ts, qst, so, f32it, f64it, reason);
        iters = f32it + f64it;
        if (outcome == FAST_REPLAY) {   // the reference's FP64 iteration from its start, in place
            us = ts = qst = 1e-4;
            surface_const(P, c, c.Ti, qs0, s);
            iters = solve_plain<false>(P, c, s, us, ts, qst, nonconv);
            f64it = iters;
            replayed = true;
            if (stats) stats_replay_reason(stats, reason);
        }
    }
    al_store(P, a, k, c, us, ts, qst, c.Ti, iters);
    if (stats) stats_add(stats, true, true, iters, nonconv, f64it > 0, f64it, replayed, false);
}

template <class S>
static cudaError_t launch_al_t(const ALArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                               SolveOpts so, DevStats* stats, cudaStream_t stream) {
    const int64_t n = (int64_t)a.L.nx * a.L.ny;
    const int block = so.block;   // <= 128: the kernel is compiled with __launch_bounds__(128)
    const unsigned grid = (unsigned)((n + block - 1) / block);
    if (prec == NESF_PLAIN_F64) al_kernel<S, NESF_PLAIN_F64><<<grid, block, 0, stream>>>(a, P64, P32, so, stats);
    else al_kernel<S, NESF_F32_POLISH><<<grid, block, 0, stream>>>(a, P64, P32, so, stats);
    cudaError_t e = cudaGetLastError();
    trace_mark(so.tracer, "al_solve", stream);
    return e;
}

// The build compiles this file once per storage type (NESF_STORAGE = 64, then 32), so the
// two halves of the kernel instantiations compile in parallel; undefined builds both.
#if !defined(NESF_STORAGE) || NESF_STORAGE == 64
cudaError_t launch_al(const ALArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, DevStats* stats, cudaStream_t stream) {
    return launch_al_t(a, P64, P32, prec, so, stats, stream);
}
#endif
#if !defined(NESF_STORAGE) || NESF_STORAGE == 32
cudaError_t launch_al(const ALArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      SolveOpts so, DevStats* stats, cudaStream_t stream) {
    return launch_al_t(a, P64, P32, prec, so, stats, stream);
}
#endif

}  // namespace nesf
