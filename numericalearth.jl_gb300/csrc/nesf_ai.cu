// nesf_ai.cu -- atmosphere-sea-ice similarity-theory solve.
//
// _compute_atmosphere_ocean_interface_state!  (InterfaceComputations/atmosphere_ocean_fluxes.jl:80-197)
// _compute_atmosphere_sea_ice_interface_state! (InterfaceComputations/atmosphere_sea_ice_fluxes.jl:65-185)
//
// One thread per surface cell over the halo ring (0:nx+1, 0:ny+1), SoA loads of
// the Oceananigans parent arrays (i fastest, so a warp reads 32 consecutive
// cells of a row). Two precisions:
//   PLAIN   every iteration in FP64 (the drop-in, parity with the CPU solver);
//   POLISH  FP64 prologue for the loop invariants, the fixed point in FP32 until
//           it converges (drift < tol) or stalls at FP32 resolution, then FP64
//           fixed-point polish steps from the FP32 state for the stalled cells.
#include "nesf_solve.cuh"

namespace nesf {

// ------------------------------------------------------------------ AI kernel
template <class S, int PREC>
__global__ void __launch_bounds__(128) ai_kernel(AIArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                 int polish_maxiter, DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= ring) return;
    int i = (int)(r % nxr), j = (int)(r / nxr);
    int64_t k = a.L.at(i, j);
    const DevIface<double>& P = P64;
    CellConst<double> c;
    c.ua = ld(a.ua, k); c.va = ld(a.va, k); c.Ta = ld(a.Ta, k); c.pa = ld(a.pa, k); c.qa = ld(a.qa, k);
    c.Ti = ld(a.To, k) + P.off_int;
    c.Si = ld(a.So, k);
    c.ui = 0; c.vi = 0;
    c.hi = ld(a.hi, k);
    c.hs = ldz(a.hs, k);
    c.hc = ld(a.hc, k);
    double aleph = ld(a.aleph, k);
    double Ts0 = ld(a.Ts, k) + P.off_ifc;
    c.sw = ldz(a.sw, k);
    c.lw = ldz(a.lw, k);
    c.kappa = -1.0;
    bool land = a.inactive ? a.inactive[k] != 0 : false;
    if (P.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    else { c.du = c.ua - 0.0; c.dv = c.va - 0.0; }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = surface_atmosphere_temperature(P, c.Ta, c.qa);
    c.rho_a = air_density(P, c.Ta, c.pa, c.qa);
    c.cp_a = cp_m(P, c.qa);
    c.L_s = latent_heat_sublim(P, c.Ta);

    double us = 1e-4, ts = 1e-4, qst = 1e-4;
    double qs0 = surface_specific_humidity(P, c.pa, Ts0);
    SurfaceConst<double> s;
    surface_const(P, c, Ts0, qs0, s);
    bool ice_free = aleph == 0;
    bool needs = P.stop_kind == NESF_STOP_CONVERGENCE;
    int iters = 0, piters = 0;
    bool nonconv = false;
    bool solved = !((needs && land) || ice_free);
    double Ts;
    if (solved) {
        if (P.temp_form == NESF_BULK_TEMPERATURE)
            iters = solve_cell<PREC, false>(P64, P32, c, s, us, ts, qst, polish_maxiter, nonconv, piters);
        else
            iters = solve_cell<PREC, true>(P64, P32, c, s, us, ts, qst, polish_maxiter, nonconv, piters);
        Ts = s.Ts;
    } else {
        us = ts = qst = 0;
        Ts = c.Ti;
    }
    double du = c.du, dv = c.dv;
    double dU = sqrt(du * du + dv * dv);
    double tx = dU == 0 ? 0.0 : -(us * us) * du / dU;
    double ty = dU == 0 ? 0.0 : -(us * us) * dv / dU;
    double rho = c.rho_a, cp = c.cp_a, Li = c.L_s;
    st(a.Qv, k, -rho * us * qst * Li);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    a.Ts[k] = (S)(Ts - P.off_ifc);
    if (a.iters) a.iters[k] = iters;
    if (stats) stats_add(stats, true, solved, iters, nonconv, piters > 0, piters, false, 0);
}

template <class S>
static cudaError_t launch_ai_t(const AIArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                               int polish_maxiter, DevStats* stats, cudaStream_t stream) {
    const int64_t ring = (int64_t)(a.L.nx + 2) * (a.L.ny + 2);
    const int block = 128;
    dim3 grid((unsigned)((ring + block - 1) / block));
    if (prec == NESF_PLAIN_F64) ai_kernel<S, NESF_PLAIN_F64><<<grid, block, 0, stream>>>(a, P64, P32, polish_maxiter, stats);
    else ai_kernel<S, NESF_F32_POLISH><<<grid, block, 0, stream>>>(a, P64, P32, polish_maxiter, stats);
    return cudaGetLastError();
}

cudaError_t launch_ai(const AIArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      int polish_maxiter, DevStats* stats, cudaStream_t stream) {
    return launch_ai_t(a, P64, P32, prec, polish_maxiter, stats, stream);
}
cudaError_t launch_ai(const AIArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32, int prec,
                      int polish_maxiter, DevStats* stats, cudaStream_t stream) {
    return launch_ai_t(a, P64, P32, prec, polish_maxiter, stats, stream);
}

}  // namespace nesf
