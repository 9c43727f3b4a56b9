// nesf_exchange.cu -- the streaming kernels of the interface-flux step:
//   sea-ice-ocean fluxes  (InterfaceComputations/sea_ice_ocean_fluxes.jl:106-226,
//                          sea_ice_ocean_heat_flux_formulations.jl:176-313)
//   fractional indices    (Atmospheres/prescribed_atmosphere_regridder.jl:51-71)
//   atmosphere + radiation interpolation (Atmospheres/interpolate_atmospheric_state.jl:91-137,
//                          Radiations/interpolate_radiation_state.jl:43-69)
//   net ocean / sea-ice flux assembly (Oceans/assemble_net_ocean_fluxes.jl:74-153,
//                          SeaIces/assemble_net_sea_ice_fluxes.jl:42-81)
//   radiative add-ons     (Radiations/apply_air_sea_radiative_fluxes.jl:62-111,
//                          Radiations/apply_air_sea_ice_radiative_fluxes.jl:55-90)
// All are HBM-bound: one thread per cell, i fastest, read-once/write-once.
#include "nesf_exchange.cuh"

#include <climits>

namespace nesf {

// ------------------------------------------------------------- sea ice - ocean
// The parameters in arithmetic R, converted once on the host: a conversion from FP64
// inside the kernel runs on the FP64 pipe, at 1/64 of the FP32 rate on this part, and
// with FP32 fields it was most of the streaming kernels' time.
template <class R> struct IOConsts {
    R rho, cpo, Tfw, slope, ht, us, st, E, kice;
};
template <class R> static IOConsts<R> io_consts(const nesf_io_params& p) {
    return IOConsts<R>{R(p.ocean_reference_density), R(p.ocean_heat_capacity),
                       R(p.liquidus_freshwater_melting_temperature), R(p.liquidus_slope),
                       R(p.heat_transfer_coefficient), R(p.friction_velocity), R(p.salt_transfer_coefficient),
                       R(p.reference_latent_heat), R(p.ice_conductivity)};
}

// The interface heat flux, temperature and salinity of one cell in arithmetic R
// (sea_ice_ocean_fluxes.jl:183-205): the bulk formulation, or the three-equation
// interface conditions (solve_interface_conditions,
// sea_ice_ocean_heat_flux_formulations.jl:280-313) with the MITgcm root choice.
template <class R, class S>
__device__ __forceinline__ void io_interface(const IOArgs<S>& a, const nesf_io_params& p, const IOConsts<R>& C,
                                             int64_t k2, R TN, R SN, S& Qio_out, S& Tb_out, S& Sb_out) {
    const R rho = C.rho, cpo = C.cpo;
    const R Tfw = C.Tfw, slope = C.slope;
    R Si = ldr<R>(a.Si, k2), h = ldr<R>(a.hi, k2), aleph = ldr<R>(a.aleph, k2), hc = ldr<R>(a.hc, k2);
    R Tsi = (p.conductive && a.Tint) ? ldr<R>(a.Tint, k2) : R(0);
    if (p.formulation == 1) {
        R Tm = Tfw - slope * SN;
        Qio_out = S(rho * cpo * C.ht * C.us * (TN - Tm) * aleph);
        Tb_out = S(Tm);
        Sb_out = S(SN);
        return;
    }
    R E = C.E;
    R kap = R(0), Ti = R(0);
    if (p.conductive) {
        kap = h >= hc ? C.kice / (h * E) : R(0);
        Ti = Tsi;
    }
    R l1 = -slope, l2 = Tfw;
    R us = C.us;
    R eta = rho * cpo * C.ht * us / E;
    R gam = rho * C.st * us;
    R th = eta + kap;
    R qa = th * l1;
    R qb = -gam - eta * TN - kap * Ti + th * (l2 - l1 * Si);
    R qc = gam * SN + (eta * TN + kap * Ti - th * l2) * Si;
    R xi = qa == R(0) ? R(0) : R(1) / (R(2) * qa);
    R D = M<R>::fmax(qb * qb - R(4) * qa * qc, R(0));   // Julia max
    R sD = M<R>::sqrt(D);
    R Ss = (-qb - sD) * xi;
    Ss = Ss < R(0) ? (-qb + sD) * xi : Ss;
    R Ts = l2 - slope * Ss;
    R q = eta * (TN - Ts) + kap * (Ti - Ts);
    Qio_out = S(E * q * aleph);
    Tb_out = S(Ts);
    Sb_out = S(Ss);
}

// Arithmetic in the storage type S, like the streaming kernels: FP64 fields as the
// reference's Float64 kernels (bit-identical to the oracle), FP32 fields as its
// Float32 ones. PART 0: the whole computation. PART 1: the fluxes alone, from the
// frazil-adjusted column temperatures held in registers, leaving T3 unchanged;
// PART 2: the frazil adjustment of T3 alone. PART 1 then PART 2 leave the same
// state as PART 0, and PART 1 only reads the ocean state, so it may run beside
// kernels that read it.
template <class S, int PART>
__global__ void __launch_bounds__(256) io_kernel(IOArgs<S> a, nesf_io_params p, IOConsts<S> C, IOConsts<df> Cdf) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)a.L.nx * a.L.ny;
    if (r >= n) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k2 = a.L.at(i, j);
    const R rho = C.rho, cpo = C.cpo;
    const R Tfw = C.Tfw, slope = C.slope;
    // Part 1: frazil over the column, top level first (sea_ice_ocean_fluxes.jl:153-181).
    // FP32 fields: T_m - T_k cancels in a freezing level, so a level whose FP32 test is
    // within a few ulps of T_m, or that freezes, is decided, adjusted and charged in FP64
    // from its FP32 values (exact in FP64); dQ accumulates in FP64.
    double dQ = 0.0;
    R TN = R(0);
    bool top_frozen = false, any_charged = false;
    for (int kk = p.nz; kk >= 1; kk--) {
        int64_t k3 = k2 + (int64_t)(kk - 1) * p.stride_k;
        R Tk = a.T3[k3], Sk = a.S3[k3];
        R Tm = Tfw - slope * Sk;
        bool freezing = Tk < Tm;
        double dE = 0.0;
        bool charged = true;
        if (sizeof(R) < sizeof(double)) {
            // (T_k - T_m is exact in FP32 when the two are that close)
            const bool near = !(M<R>::fabs(Tk - Tm) > R(4.0 * 1.1920929e-7) * M<R>::fabs(Tm));
            charged = freezing || near;
            if (charged) {
                const double Tm64 = p.liquidus_freshwater_melting_temperature - p.liquidus_slope * (double)Sk;
                freezing = (double)Tk < Tm64;
                Tm = (R)Tm64;
                dE = (freezing ? 1.0 : 0.0) * p.ocean_reference_density * p.ocean_heat_capacity *
                     (Tm64 - (double)Tk);
            }
        } else {
            dE = (double)((freezing ? R(1) : R(0)) * rho * cpo * (Tm - Tk));
        }
        if (PART != 1 && freezing) a.T3[k3] = Tm;
        if (PART == 2) continue;
        if (sizeof(R) < sizeof(double)) {
            if (charged) dQ -= dE * a.dz[kk - 1] / p.dt;
            any_charged = any_charged || charged;
        } else {
            dQ = (double)((R)dQ - (R)dE * R(a.dz[kk - 1]) / R(p.dt));
        }
        if (kk == p.nz) {                         // the top level after the adjustment
            TN = freezing ? Tm : Tk;
            top_frozen = freezing;
        }
    }
    if (PART == 2) return;
    // FP32 fields: dQ is still its +0 unless a level was charged (no FP64 conversion then)
    st(a.frazil, k2, (sizeof(R) < sizeof(double) && !any_charged) ? R(0) : (R)dQ);
    int64_t kN = k2 + (int64_t)(p.nz - 1) * p.stride_k;
    R SN = a.S3[kN];
    R aleph = ldr<R>(a.aleph, k2);
    R Qio, Tb, Sb;
    // FP32 fields: where the ice covers part of the cell, the interface heat
    // eta (T_N - T_b) + kappa (T_i - T_b) cancels near the melting point and would
    // multiply FP32's rounding of S_b by |T_b| / |T_N - T_b|; the interface
    // conditions are solved in double-float there (48 bits, on the FP32 pipes: FP64
    // issues one warp instruction per ~64 cycles per SM sub-partition on this GPU),
    // from the FP32 inputs (exact in double-float), with a frozen top level at its
    // melting point T_m(S_N) in double-float.
    if (sizeof(S) < sizeof(double) && aleph > R(0)) {
        const df SNd((float)SN);
        const df TNd = top_frozen ? Cdf.Tfw - Cdf.slope * SNd : df((float)TN);
        io_interface<df>(a, p, Cdf, k2, TNd, SNd, Qio, Tb, Sb);
    } else {
        io_interface<R>(a, p, C, k2, TN, SN, Qio, Tb, Sb);
    }
    if (p.formulation != 1) {
        st(a.Tb, k2, Tb);
        st(a.Sb, k2, Sb);
    }
    st(a.Qio, k2, Qio);
    R Si = ldr<R>(a.Si, k2);
    R Ei = ldzr<R>(a.Ei, k2), Es = ldzr<R>(a.Es, k2);
    st(a.Jw, k2, -(Ei + Es) / rho);
    st(a.Js, k2, Ei * Si / rho);
}

// ---------------------------------------------------------- fractional indices
__global__ void frac_kernel(Layout2 L, nesf_exchange_coords c, nesf_atmos_grid ag, double* fi, double* fj) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int wx = L.nx + 2 * L.hx, wy = L.ny + 2 * L.hy;
    if (r >= (int64_t)wx * wy) return;
    int i = 1 - L.hx + (int)(r % wx), j = 1 - L.hy + (int)(r / wx);
    int64_t k = L.at(i, j);
    double lon = c.lon0 + (i - 1) * c.dlon;
    double lat = c.lat0 + (j - 1) * c.dlat;
    fi[k] = (lon - ag.lon0) / ag.dlon + 1;
    fj[k] = (lat - ag.lat0) / ag.dlat + 1;
}

// ------------------------------------------------------------- interpolation
// Arithmetic in the storage type S: FP64 fields interpolate exactly as the
// reference's Float64 kernels, FP32 fields as its Float32 ones (the weights from
// the FP64 fractional indices, rounded once).
template <class S>
__device__ __forceinline__ S interp_one(const nesf_atmos_grid& ag, const S* __restrict__ d, int i0, int i1, int j0,
                                        int j1, S xi, S eta, S tn) {
    S v[2];
#pragma unroll
    for (int n = 0; n < 2; n++) {
        const S* b = d + (int64_t)n * ag.stride_t;
        auto at = [&](int ii, int jj) {
            return __ldg(b + (int64_t)(ii - 1 + ag.hx) + (int64_t)(jj - 1 + ag.hy) * ag.stride_j);
        };
        v[n] = (1 - xi) * (1 - eta) * at(i0, j0) + (1 - xi) * eta * at(i0, j1) + xi * (1 - eta) * at(i1, j0) +
               xi * eta * at(i1, j1);
    }
    return v[1] * tn + v[0] * (1 - tn);
}

__device__ __forceinline__ int wrap_i(int i, int n) {
    int m = (i - 1) % n;
    if (m < 0) m += n;
    return m + 1;
}
__device__ __forceinline__ int clamp_j(int j, int n) { return j < 1 ? 1 : (j > n ? n : j); }

template <class S>
__global__ void __launch_bounds__(256) interp_kernel(InterpArgs<S> a) {
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int nxr = a.L.nx + 2;
    if (r >= (int64_t)nxr * (a.L.ny + 2)) return;
    int i = (int)(r % nxr), j = (int)(r / nxr);
    int64_t k = a.L.at(i, j);
    double fi, fj;
    if (a.frac_i) {
        fi = a.frac_i[k];
        fj = a.frac_j[k];
    } else {
        double lon = a.coords.lon0 + (i - 1) * a.coords.dlon;
        double lat = a.coords.lat0 + (j - 1) * a.coords.dlat;
        fi = (lon - a.atmos.lon0) / a.atmos.dlon + 1;
        fj = (lat - a.atmos.lat0) / a.atmos.dlat + 1;
    }
    double fli = floor(fi), flj = floor(fj);
    int im = (int)fli, jm = (int)flj;
    S xi = (S)(fi - fli), eta = (S)(fj - flj);
    int i0 = wrap_i(im, a.atmos.nx), i1 = wrap_i(im + 1, a.atmos.nx);
    int j0 = clamp_j(jm, a.atmos.ny), j1 = clamp_j(jm + 1, a.atmos.ny);
    const S tn = (S)a.tn;
#pragma unroll
    for (int n = 0; n < 9; n++) {
        if (!a.dst[n]) continue;
        a.dst[n][k] = a.src[n] ? interp_one<S>(a.atmos, a.src[n], i0, i1, j0, j1, xi, eta, tn) : S(0);
    }
}

// Tiled interpolation for a regular longitude-latitude exchange grid without fractional
// index caches: a block of 256 threads covers 256 ring columns x tile_rows ring rows. The
// fractional indices depend on the column (longitude) and on the row (latitude) alone, so
// the block computes them once per column and once per row, in FP64 with the gather
// kernel's expressions (the same values), and stages the coarse footprint of its tile --
// the atmosphere columns and rows its cells' bilinear stencils touch, both snapshots of
// all nine variables -- in shared memory with coalesced loads; each cell then reads its
// four corners there. The interpolation arithmetic is the gather kernel's (same
// expressions, same order: bit-identical outputs). A tile whose footprint would exceed
// the staged bounds (fp_w x fp_h, sized on the host) reads its corners from global memory.
constexpr int kInterpTileCols = 256;
constexpr int kInterpTileRows = 16;      // rows of a tile unless one wave of taller tiles covers the grid
constexpr int kInterpMaxTileRows = 32;

template <class S>
__global__ void __launch_bounds__(kInterpTileCols) interp_tile_kernel(InterpArgs<S> a) {
    extern __shared__ __align__(16) unsigned char interp_smem[];
    S* stage = (S*)interp_smem;
    __shared__ int s_jm[kInterpMaxTileRows];
    __shared__ S s_eta[kInterpMaxTileRows];
    __shared__ int s_bounds[4];   // smallest and largest stencil column (unwrapped), row (clamped)
    const int nxr = a.L.nx + 2, nyr = a.L.ny + 2;
    const nesf_atmos_grid& ag = a.atmos;
    const int i = blockIdx.x * kInterpTileCols + threadIdx.x;   // ring column 0..nx+1
    const int jt = blockIdx.y * a.tile_rows;                     // first ring row of the tile
    const int nj = min(a.tile_rows, nyr - jt);
    const bool col = i < nxr;
    int im = 0;
    S xi = S(0);
    if (col) {
        double lon = a.coords.lon0 + (i - 1) * a.coords.dlon;
        double fi = (lon - ag.lon0) / ag.dlon + 1;
        double fli = floor(fi);
        // |fi| beyond 2^28 means coordinates far outside the atmosphere's: the clamp keeps the
        // footprint arithmetic below from overflowing (wrap_i gives such cells a column anyway)
        im = (int)fmin(fmax(fli, -268435456.0), 268435456.0);
        xi = (S)(fi - fli);
    }
    if (threadIdx.x == 0) {
        s_bounds[0] = INT_MAX; s_bounds[1] = INT_MIN; s_bounds[2] = INT_MAX; s_bounds[3] = INT_MIN;
    }
    __syncthreads();
    if (threadIdx.x < nj) {
        int j = jt + threadIdx.x;
        double lat = a.coords.lat0 + (j - 1) * a.coords.dlat;
        double fj = (lat - ag.lat0) / ag.dlat + 1;
        double flj = floor(fj);
        int jm = (int)flj;
        s_jm[threadIdx.x] = jm;
        s_eta[threadIdx.x] = (S)(fj - flj);
        atomicMin(&s_bounds[2], clamp_j(jm, ag.ny));
        atomicMax(&s_bounds[3], clamp_j(jm + 1, ag.ny));
    }
    if (col) {
        atomicMin(&s_bounds[0], im);
        atomicMax(&s_bounds[1], im + 1);
    }
    __syncthreads();
    const int imin = s_bounds[0], jmin = s_bounds[2];
    const int64_t W64 = (int64_t)s_bounds[1] - imin + 1, H64 = (int64_t)s_bounds[3] - jmin + 1;
    const bool staged = W64 >= 2 && H64 >= 1 && W64 <= a.fp_w && H64 <= a.fp_h;   // block-uniform
    const int W = staged ? (int)W64 : 0, H = staged ? (int)H64 : 0;
    const int plane = W * H;
    if (staged) {
        // one (row, column) per element of the footprint, the 18 planes (variable, snapshot) in turn
        for (int e = threadIdx.x; e < plane; e += kInterpTileCols) {
            const int r = e / W, c = e - r * W;
            const int64_t at = (int64_t)(wrap_i(imin + c, ag.nx) - 1 + ag.hx) + (int64_t)(jmin + r - 1 + ag.hy) * ag.stride_j;
#pragma unroll
            for (int q = 0; q < 18; q++) {
                const S* b = a.src[q >> 1];
                stage[q * plane + e] = b ? __ldg(b + (int64_t)(q & 1) * ag.stride_t + at) : S(0);
            }
        }
    }
    __syncthreads();
    if (!col) return;
    const int i0 = wrap_i(im, ag.nx), i1 = wrap_i(im + 1, ag.nx);
    const int c0 = im - imin, c1 = c0 + 1;
    const S tn = (S)a.tn;
    for (int r = 0; r < nj; r++) {
        const int j = jt + r;
        const int jm = s_jm[r];
        const S eta = s_eta[r];
        const int j0 = clamp_j(jm, ag.ny), j1 = clamp_j(jm + 1, ag.ny);
        const int64_t k = a.L.at(i, j);
        if (staged) {
            const int r0 = j0 - jmin, r1 = j1 - jmin;
#pragma unroll
            for (int n = 0; n < 9; n++) {
                if (!a.dst[n]) continue;
                S out = S(0);
                if (a.src[n]) {
                    S v[2];
#pragma unroll
                    for (int t = 0; t < 2; t++) {
                        const S* q = stage + (2 * n + t) * plane;
                        auto at = [&](int cc, int rr) { return q[rr * W + cc]; };
                        v[t] = (1 - xi) * (1 - eta) * at(c0, r0) + (1 - xi) * eta * at(c0, r1) +
                               xi * (1 - eta) * at(c1, r0) + xi * eta * at(c1, r1);
                    }
                    out = v[1] * tn + v[0] * (1 - tn);
                }
                a.dst[n][k] = out;
            }
        } else {
#pragma unroll
            for (int n = 0; n < 9; n++) {
                if (!a.dst[n]) continue;
                a.dst[n][k] = a.src[n] ? interp_one<S>(ag, a.src[n], i0, i1, j0, j1, xi, eta, tn) : S(0);
            }
        }
    }
}

// ------------------------------------------------------------------ assembly
// Arithmetic in the storage type S, as the interpolation; the parameters converted to S
// once on the host (as the sea-ice-ocean kernel's).
template <class R> struct AsmConsts {
    R rho, cpo, off, sigma, eps_o, alb_o, eps_i, alb_i;
};
template <class R> static AsmConsts<R> asm_consts(const nesf_assembly_params& p) {
    return AsmConsts<R>{R(p.ocean_reference_density), R(p.ocean_heat_capacity), R(p.interface_temperature_offset),
                        R(p.stefan_boltzmann_constant), R(p.ocean_emissivity), R(p.ocean_albedo),
                        R(p.ice_emissivity), R(p.ice_albedo)};
}

template <class S>
__global__ void __launch_bounds__(256) assemble_ocean_kernel(AsmArgs<S> a, AsmConsts<S> p) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k = a.L.at(i, j), kw = k - 1, ks = k - a.L.sj;
    const R rinv = R(1) / p.rho;
    const R cinv = R(1) / p.cpo;
    R al = ldzr<R>(a.f.aleph, k);
    R To = ldr<R>(a.f.To, k);
    R Jr = ldzr<R>(a.f.rain, k), Js = ldzr<R>(a.f.snow, k), Ps = ldzr<R>(a.f.isnow, k), Jl = ldzr<R>(a.f.land_fw, k);
    R QT = ldr<R>(a.f.ao_QT, k), Qv = ldr<R>(a.f.ao_Qv, k), Jv = ldr<R>(a.f.ao_Jv, k);
    R SQao = (QT + Qv) * (1 - al);
    R SFao = -(Jr + Jl + Js - Ps) * rinv + (1 - al) * Jv * rinv;
    R Jwao = -SFao;
    bool inactive = a.f.inactive ? a.f.inactive[k] != 0 : false;
    R Qin = ldzr<R>(a.f.io_Q, k), Jsio = ldzr<R>(a.f.io_Js, k), Jwio = ldzr<R>(a.f.io_Jw, k);
    R JTao = SQao * rinv * cinv;
    R JTio = Qin * rinv * cinv;
    R aw = ldzr<R>(a.f.aleph, kw), as = ldzr<R>(a.f.aleph, ks);
    R tcx = rinv * (1 - al) * ldr<R>(a.f.ao_tx, k);
    R tcxw = rinv * (1 - aw) * ldr<R>(a.f.ao_tx, kw);
    R tcy = rinv * (1 - al) * ldr<R>(a.f.ao_ty, k);
    R tcys = rinv * (1 - as) * ldr<R>(a.f.ao_ty, ks);
    R txao = (tcxw + tcx) / 2;
    R tyao = (tcys + tcy) / 2;
    R txio = ldzr<R>(a.f.io_tx, k) * rinv * ((aw + al) / 2);
    R tyio = ldzr<R>(a.f.io_ty, k) * rinv * ((as + al) / 2);
    st(a.f.o_u, k, inactive ? R(0) : txao + txio);
    st(a.f.o_v, k, inactive ? R(0) : tyao + tyio);
    R JT = inactive ? R(0) : JTao + JTio;
    if (a.with_radiation) {
        // apply_air_sea_radiative_fluxes fused: J_T += radiative part
        R Ts = ldr<R>(a.f.ao_Ts, k) + p.off;
        R T2 = Ts * Ts;
        R Iup = p.sigma * p.eps_o * (T2 * T2);
        R Ia = -p.eps_o * ldr<R>(a.f.lw, k);
        R It = -(1 - p.alb_o) * ldr<R>(a.f.sw, k);
        Ia *= (1 - al);
        It *= (1 - al);
        R Iup_o = Iup * (1 - al);
        R SQ = Iup_o + Ia + It;
        R JTr = SQ * rinv * cinv;
        JT += inactive ? R(0) : JTr;
        st(a.f.o_up_lw, k, Iup);
        st(a.f.o_dn_lw, k, -Ia);
        st(a.f.o_dn_sw, k, -It);
    }
    st(a.f.o_T, k, JT);
    st(a.f.o_S, k, inactive ? R(0) : Jsio);
    st(a.f.o_eta, k, inactive ? R(0) : Jwao + Jwio);
    st(a.f.o_H, k, inactive ? R(0) : To * Jwao);
}

template <class S>
__global__ void __launch_bounds__(256) assemble_ice_kernel(AsmArgs<S> a, AsmConsts<S> p) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k = a.L.at(i, j), kw = k - 1, ks = k - a.L.sj;
    R al = ldr<R>(a.f.aleph, k);
    R QT = ldr<R>(a.f.ai_QT, k), Qv = ldr<R>(a.f.ai_Qv, k);
    R Qf = ldzr<R>(a.f.io_Qf, k), Qi = ldzr<R>(a.f.io_Q, k);
    R Js = ldzr<R>(a.f.snow, k);
    R SQt = (QT + Qv) * al;
    R SQb = Qf + Qi;
    bool inactive = a.f.inactive ? a.f.inactive[k] != 0 : false;
    R top = inactive ? R(0) : SQt;
    if (a.with_radiation) {
        R Ts = ldr<R>(a.f.ai_Ts, k) + p.off;
        R T2 = Ts * Ts;
        R Iup = p.sigma * p.eps_i * (T2 * T2);
        R Ia = -p.eps_i * ldr<R>(a.f.lw, k);
        R It = -(1 - p.alb_i) * ldr<R>(a.f.sw, k);
        R SQ = (Iup + Ia + It) * al;
        top += inactive ? R(0) : SQ;
        st(a.f.i_up_lw, k, Iup);
        st(a.f.i_dn_lw, k, -Ia);
        st(a.f.i_dn_sw, k, -It);
    }
    st(a.f.i_top, k, top);
    st(a.f.i_snow, k, inactive ? R(0) : Js);
    st(a.f.i_u, k, inactive ? R(0) : (ldr<R>(a.f.ai_tx, kw) + ldr<R>(a.f.ai_tx, k)) / 2);
    st(a.f.i_v, k, inactive ? R(0) : (ldr<R>(a.f.ai_ty, ks) + ldr<R>(a.f.ai_ty, k)) / 2);
    st(a.f.i_bottom, k, inactive ? R(0) : SQb);
}

// Radiation alone, added in place to an already assembled J_T / top heat flux.
template <class S, bool ICE>
__global__ void __launch_bounds__(256) radiation_kernel(AsmArgs<S> a, AsmConsts<S> p) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k = a.L.at(i, j);
    bool inactive = a.f.inactive ? a.f.inactive[k] != 0 : false;
    if (!ICE) {
        const R rinv = R(1) / p.rho, cinv = R(1) / p.cpo;
        R al = ldzr<R>(a.f.aleph, k);
        R Ts = ldr<R>(a.f.ao_Ts, k) + p.off;
        R T2 = Ts * Ts;
        R Iup = p.sigma * p.eps_o * (T2 * T2);
        R Ia = -p.eps_o * ldr<R>(a.f.lw, k);
        R It = -(1 - p.alb_o) * ldr<R>(a.f.sw, k);
        Ia *= (1 - al);
        It *= (1 - al);
        R Iup_o = Iup * (1 - al);
        R SQ = Iup_o + Ia + It;
        R JT = SQ * rinv * cinv;
        a.f.o_T[k] = a.f.o_T[k] + (inactive ? R(0) : JT);
        st(a.f.o_up_lw, k, Iup);
        st(a.f.o_dn_lw, k, -Ia);
        st(a.f.o_dn_sw, k, -It);
    } else {
        R al = ldr<R>(a.f.aleph, k);
        R Ts = ldr<R>(a.f.ai_Ts, k) + p.off;
        R T2 = Ts * Ts;
        R Iup = p.sigma * p.eps_i * (T2 * T2);
        R Ia = -p.eps_i * ldr<R>(a.f.lw, k);
        R It = -(1 - p.alb_i) * ldr<R>(a.f.sw, k);
        R SQ = (Iup + Ia + It) * al;
        a.f.i_top[k] = a.f.i_top[k] + (inactive ? R(0) : SQ);
        st(a.f.i_up_lw, k, Iup);
        st(a.f.i_dn_lw, k, -Ia);
        st(a.f.i_dn_sw, k, -It);
    }
}

// _assemble_slab_land_fluxes! (Lands/slab_land.jl:316-329): every interior cell of the land
// grid, masked or not, as the reference writes them.
template <class S>
__global__ void __launch_bounds__(256) land_assemble_kernel(LandArgs<S> a) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k = a.L.at(i, j);
    R QT = ldr<R>(a.QT, k), Qv = ldr<R>(a.Qv, k), Jv = ldr<R>(a.Jv, k);
    R rain = ldzr<R>(a.rain, k);
    st(a.Es, k, QT + Qv);
    st(a.P, k, rain + M<R>::fmax(R(0), -Jv));
    st(a.E, k, M<R>::fmax(R(0), Jv));
    st(a.Jvo, k, Jv);
    st(a.Pl, k, rain);
}

// _apply_air_land_radiative_fluxes! (Radiations/apply_air_land_radiative_fluxes.jl:60-95):
// sum_rad = -sigma eps T^4 - (-eps LW - (1 - alpha) SW), positive into the land, enters the
// upward surface_energy_flux with its sign flipped.
template <class S>
__global__ void __launch_bounds__(256) land_radiation_kernel(LandArgs<S> a, nesf_land_radiation_params p) {
    using R = S;
    int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= (int64_t)a.L.nx * a.L.ny) return;
    int i = 1 + (int)(r % a.L.nx), j = 1 + (int)(r / a.L.nx);
    int64_t k = a.L.at(i, j);
    R Ts = ldr<R>(a.Ts, k);
    R T2 = Ts * Ts;
    R Iup = R(p.stefan_boltzmann_constant) * R(p.land_emissivity) * (T2 * T2);
    R Ia = -R(p.land_emissivity) * ldr<R>(a.lw, k);
    R It = -(1 - R(p.land_albedo)) * ldr<R>(a.sw, k);
    R SQ = -Iup - (Ia + It);
    bool inactive = a.inactive ? a.inactive[k] != 0 : false;
    a.Es[k] = a.Es[k] + (inactive ? R(0) : -SQ);
    st(a.up_lw, k, Iup);
    st(a.dn_lw, k, -Ia);
    st(a.dn_sw, k, -It);
}

// ------------------------------------------------------------------ launchers
static inline unsigned blocks_for(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

template <class S>
cudaError_t launch_io(const IOArgs<S>& a, const nesf_io_params& p, cudaStream_t s, int part) {
    int64_t n = (int64_t)a.L.nx * a.L.ny;
    const IOConsts<S> C = io_consts<S>(p);
    const IOConsts<df> Cdf = io_consts<df>(p);
    if (part == 1) io_kernel<S, 1><<<blocks_for(n, 256), 256, 0, s>>>(a, p, C, Cdf);
    else if (part == 2) io_kernel<S, 2><<<blocks_for(n, 256), 256, 0, s>>>(a, p, C, Cdf);
    else io_kernel<S, 0><<<blocks_for(n, 256), 256, 0, s>>>(a, p, C, Cdf);
    return cudaGetLastError();
}
template cudaError_t launch_io<double>(const IOArgs<double>&, const nesf_io_params&, cudaStream_t, int);
template cudaError_t launch_io<float>(const IOArgs<float>&, const nesf_io_params&, cudaStream_t, int);

cudaError_t launch_frac(const Layout2& L, const nesf_exchange_coords& c, const nesf_atmos_grid& ag, double* fi,
                        double* fj, cudaStream_t s) {
    int64_t n = (int64_t)(L.nx + 2 * L.hx) * (L.ny + 2 * L.hy);
    frac_kernel<<<blocks_for(n, 256), 256, 0, s>>>(L, c, ag, fi, fj);
    return cudaGetLastError();
}

// The tiled kernel serves a regular grid without caches when a tile's coarse footprint fits
// in kInterpStageBytes of shared memory: tile rows are halved from kInterpTileRows until
// it does (the per-cell gather kernel otherwise). Footprint bounds: a tile's columns span
// (kInterpTileCols - 1) |dlon / dlon_atmos| fractional indices, its rows (rows - 1) |dlat /
// dlat_atmos|; + 1 for the stencil's second point and + 1 for the floors.
// Wave: a tile's blocks run their phases (indices, staging, outputs) one after the other,
// so a grid slightly larger than the blocks that fit on the GPU at once leaves a second
// wave of a few blocks, each alone on its SM, after the first. Where tiles of up to
// kInterpMaxTileRows rows fit the grid into one wave (and their footprint into shared
// memory), the rows are the fewest that do.
constexpr size_t kInterpStageBytes = 64 * 1024;

template <class S>
static bool interp_footprint(const InterpArgs<S>& a, int rows, int& w, int& h) {
    const double rx = fabs(a.coords.dlon / a.atmos.dlon), ry = fabs(a.coords.dlat / a.atmos.dlat);
    const double fw = ceil((kInterpTileCols - 1) * rx) + 3, fh = ceil((rows - 1) * ry) + 3;
    if (!(fw <= 4096 && fh <= 4096 && 18.0 * fw * fh * sizeof(S) <= (double)kInterpStageBytes)) return false;
    w = (int)fw;
    h = (int)fh;
    return true;
}

template <class S>
cudaError_t launch_interp(const InterpArgs<S>& a0, cudaStream_t s) {
    InterpArgs<S> a = a0;
    a.tile_rows = a.fp_w = a.fp_h = 0;
    const int64_t nyr = a.L.ny + 2;
    if (!a.frac_i) {
        int w = 0, h = 0;
        for (int rows = kInterpTileRows; rows >= 1 && !a.tile_rows; rows /= 2)
            if (interp_footprint(a, rows, w, h)) { a.tile_rows = rows; a.fp_w = w; a.fp_h = h; }
        if (a.tile_rows == kInterpTileRows) {
            cudaError_t e = cudaFuncSetAttribute(interp_tile_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kInterpStageBytes);
            if (e != cudaSuccess) return e;
            int dev = 0, sms = 0, per_sm = 0;
            const int64_t col_tiles = (a.L.nx + 2 + kInterpTileCols - 1) / kInterpTileCols;
            if (cudaGetDevice(&dev) == cudaSuccess &&
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) {
                for (int rows = kInterpTileRows; rows <= kInterpMaxTileRows; rows++) {
                    if (!interp_footprint(a, rows, w, h)) break;
                    const size_t bytes = (size_t)18 * w * h * sizeof(S);
                    if (cudaOccupancyMaxActiveBlocksPerMultiprocessorWithFlags(
                            &per_sm, interp_tile_kernel<S>, kInterpTileCols, bytes, cudaOccupancyDefault) !=
                        cudaSuccess) {
                        (void)cudaGetLastError();
                        break;
                    }
                    if (col_tiles * ((nyr + rows - 1) / rows) <= (int64_t)per_sm * sms) {
                        a.tile_rows = rows; a.fp_w = w; a.fp_h = h;
                        break;
                    }
                }
            }
        }
    }
    if (!a.tile_rows) {
        int64_t n = (int64_t)(a.L.nx + 2) * nyr;
        interp_kernel<S><<<blocks_for(n, 256), 256, 0, s>>>(a);
        return cudaGetLastError();
    }
    const size_t bytes = (size_t)18 * a.fp_w * a.fp_h * sizeof(S);
    cudaError_t e = cudaFuncSetAttribute(interp_tile_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kInterpStageBytes);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((a.L.nx + 2 + kInterpTileCols - 1) / kInterpTileCols),
              (unsigned)((nyr + a.tile_rows - 1) / a.tile_rows));
    interp_tile_kernel<S><<<grid, kInterpTileCols, bytes, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_interp<double>(const InterpArgs<double>&, cudaStream_t);
template cudaError_t launch_interp<float>(const InterpArgs<float>&, cudaStream_t);

bool is_interp_kernel(const void* fn, bool fp64) {
    return fp64 ? (fn == (const void*)interp_kernel<double> || fn == (const void*)interp_tile_kernel<double>)
                : (fn == (const void*)interp_kernel<float> || fn == (const void*)interp_tile_kernel<float>);
}

template <class S>
cudaError_t launch_assemble(const AsmArgs<S>& a, const nesf_assembly_params& p, int which, cudaStream_t s) {
    int64_t n = (int64_t)a.L.nx * a.L.ny;
    const AsmConsts<S> C = asm_consts<S>(p);
    switch (which) {
    case 0: assemble_ocean_kernel<S><<<blocks_for(n, 256), 256, 0, s>>>(a, C); break;
    case 1: assemble_ice_kernel<S><<<blocks_for(n, 256), 256, 0, s>>>(a, C); break;
    case 2: radiation_kernel<S, false><<<blocks_for(n, 256), 256, 0, s>>>(a, C); break;
    default: radiation_kernel<S, true><<<blocks_for(n, 256), 256, 0, s>>>(a, C); break;
    }
    return cudaGetLastError();
}
template cudaError_t launch_assemble<double>(const AsmArgs<double>&, const nesf_assembly_params&, int, cudaStream_t);
template cudaError_t launch_assemble<float>(const AsmArgs<float>&, const nesf_assembly_params&, int, cudaStream_t);

template <class S>
cudaError_t launch_land(const LandArgs<S>& a, const nesf_land_radiation_params& p, bool radiation, cudaStream_t s) {
    int64_t n = (int64_t)a.L.nx * a.L.ny;
    if (radiation) land_radiation_kernel<S><<<blocks_for(n, 256), 256, 0, s>>>(a, p);
    else land_assemble_kernel<S><<<blocks_for(n, 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_land<double>(const LandArgs<double>&, const nesf_land_radiation_params&, bool, cudaStream_t);
template cudaError_t launch_land<float>(const LandArgs<float>&, const nesf_land_radiation_params&, bool, cudaStream_t);

}  // namespace nesf
