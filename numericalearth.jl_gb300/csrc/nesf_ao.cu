// nesf_ao.cu -- atmosphere-ocean similarity-theory solve.
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

// ------------------------------------------------------------------ AO kernel
template <class S, int PREC, bool SKIN>
__device__ __forceinline__ void ao_cell(const DevIface<double>& P64, const DevIface<float>& P32, const AOArgs<S>& a,
                                        int i, int j, int64_t moff, int polish_maxiter, DevStats* stats) {
    const Layout2& L = a.L;
    int64_t k = L.at(i, j) + moff;
    CellConst<double> c;
    c.ua = ld(a.ua, k); c.va = ld(a.va, k); c.Ta = ld(a.Ta, k); c.pa = ld(a.pa, k); c.qa = ld(a.qa, k);
    // assemble_interior_state: centre averages of the face velocities (atmosphere_ocean_fluxes.jl:62-71)
    c.ui = (ld(a.uo, k) + ld(a.uo, k + 1)) / 2;
    c.vi = (ld(a.vo, k) + ld(a.vo, k + L.sj)) / 2;
    c.Ti = ld(a.To, k) + P64.off_int;
    c.Si = ld(a.So, k);
    c.hi = c.hs = c.hc = 0;
    c.sw = ldz(a.sw, k);
    c.lw = ldz(a.lw, k);
    c.kappa = a.kappa ? ld(a.kappa, k) : -1.0;
    bool land = a.inactive ? a.inactive[k] != 0 : false;
    if (P64.vel_form == NESF_WIND_VELOCITY) { c.du = c.ua; c.dv = c.va; }
    else { c.du = c.ua - c.ui; c.dv = c.va - c.vi; }
    c.dU2 = c.du * c.du + c.dv * c.dv;
    c.tha = surface_atmosphere_temperature(P64, c.Ta, c.qa);
    if (SKIN) {
        c.rho_a = air_density(P64, c.Ta, c.pa, c.qa);
        c.cp_a = cp_m(P64, c.qa);
        c.L_s = latent_heat_sublim(P64, c.Ta);
    } else {
        c.rho_a = c.cp_a = c.L_s = 0;
    }

    double us = 1e-4, ts = 1e-4, qst = 1e-4;
    double qs0 = surface_specific_humidity(P64, c.pa, c.Ti);
    SurfaceConst<double> s;
    surface_const(P64, c, c.Ti, qs0, s);
    bool needs = P64.stop_kind == NESF_STOP_CONVERGENCE;
    int iters = 0, piters = 0;
    bool nonconv = false;
    bool solved = !(needs && land);
    if (solved) iters = solve_cell<PREC, SKIN>(P64, P32, c, s, us, ts, qst, polish_maxiter, nonconv, piters);
    double Ts = s.Ts, ui = c.ui, vi = c.vi;
    if (land) {   // zero_interface_state (interface_states.jl:800-803)
        us = ts = qst = 0;
        Ts = 273.15;
        ui = vi = 0;
    }
    double du, dv;
    if (P64.vel_form == NESF_WIND_VELOCITY) { du = c.ua; dv = c.va; }
    else { du = c.ua - ui; dv = c.va - vi; }
    double dU = sqrt(du * du + dv * dv);
    double tx = dU == 0 ? 0.0 : -(us * us) * du / dU;
    double ty = dU == 0 ? 0.0 : -(us * us) * dv / dU;
    double rho = air_density(P64, c.Ta, c.pa, c.qa);
    double cp = cp_m(P64, c.qa);
    double Lv = latent_heat_vapor(P64, c.Ta);
    st(a.Qv, k, -rho * Lv * us * qst);
    st(a.QT, k, -rho * cp * us * ts);
    st(a.Jv, k, -rho * us * qst);
    st(a.tx, k, rho * tx);
    st(a.ty, k, rho * ty);
    st(a.Ts, k, Ts - P64.off_ifc);
    st(a.us, k, us);
    st(a.ts, k, ts);
    st(a.qs, k, qst);
    if (a.iters) a.iters[k] = iters;
    if (stats) stats_add(stats, true, solved, iters, nonconv, piters > 0, piters, false, 0);
}

template <class S, int PREC, bool SKIN, bool ENS>
__global__ void __launch_bounds__(128, ENS ? 4 : 1) ao_kernel(AOArgs<S> a, DevIface<double> P64, DevIface<float> P32,
                                                 const DevIface<double>* __restrict__ P64s,
                                                 const DevIface<float>* __restrict__ P32s, int polish_maxiter,
                                                 DevStats* stats) {
    const int nxr = a.L.nx + 2;
    const int64_t ring = (int64_t)nxr * (a.L.ny + 2);
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (ENS) {
        __shared__ DevIface<double> sP64;
        __shared__ DevIface<float> sP32;
        int m = blockIdx.y;
        if (threadIdx.x == 0) {
            sP64 = P64s[m];
            sP32 = P32s[m];
        }
        __syncthreads();
        if (r < ring) {
            int i = (int)(r % nxr), j = (int)(r / nxr);
            ao_cell<S, PREC, SKIN>(sP64, sP32, a, i, j, (int64_t)m * a.member_stride, polish_maxiter, stats);
        }
    } else {
        if (r < ring) {
            int i = (int)(r % nxr), j = (int)(r / nxr);
            ao_cell<S, PREC, SKIN>(P64, P32, a, i, j, 0, polish_maxiter, stats);
        }
    }
}

template <class S>
static cudaError_t launch_ao_t(const AOArgs<S>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                               const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec,
                               bool skin, int polish_maxiter, DevStats* stats, int block, cudaStream_t stream) {
    const int64_t ring = (int64_t)(a.L.nx + 2) * (a.L.ny + 2);
    if (block <= 0) block = 128;
    block = 128;   // kernels are compiled with __launch_bounds__(128)
    dim3 grid((unsigned)((ring + block - 1) / block), members > 1 ? members : 1);
    bool ens = members > 1 || P64s != nullptr;
#define NESF_AO_LAUNCH(PR, SK, EN) \
    ao_kernel<S, PR, SK, EN><<<grid, block, 0, stream>>>(a, P64, P32, P64s, P32s, polish_maxiter, stats)
#define NESF_AO_ENS(PR, SK) \
    do { if (ens) NESF_AO_LAUNCH(PR, SK, true); else NESF_AO_LAUNCH(PR, SK, false); } while (0)
#define NESF_AO_SKIN(PR) \
    do { if (skin) NESF_AO_ENS(PR, true); else NESF_AO_ENS(PR, false); } while (0)
    if (prec == NESF_PLAIN_F64) NESF_AO_SKIN(NESF_PLAIN_F64);
    else NESF_AO_SKIN(NESF_F32_POLISH);
#undef NESF_AO_SKIN
#undef NESF_AO_ENS
#undef NESF_AO_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_ao(const AOArgs<double>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      int polish_maxiter, DevStats* stats, int block, cudaStream_t stream) {
    return launch_ao_t(a, P64, P32, P64s, P32s, members, prec, skin, polish_maxiter, stats, block, stream);
}
cudaError_t launch_ao(const AOArgs<float>& a, const DevIface<double>& P64, const DevIface<float>& P32,
                      const DevIface<double>* P64s, const DevIface<float>* P32s, int members, int prec, bool skin,
                      int polish_maxiter, DevStats* stats, int block, cudaStream_t stream) {
    return launch_ao_t(a, P64, P32, P64s, P32s, members, prec, skin, polish_maxiter, stats, block, stream);
}

}  // namespace nesf
