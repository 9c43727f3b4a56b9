// nesf_exchange.cuh -- argument bundles of the streaming kernels (sea-ice-ocean
// fluxes, interpolation, assembly, radiation).
#pragma once

#include "nesf_kernels.cuh"

namespace nesf {

template <class S> struct IOArgs {
    Layout2 L;
    S* T3;                    // 3-D ocean temperature (level 1 pointer), mutated by frazil
    const S* S3;              // 3-D ocean salinity
    const double* dz;         // nz layer thicknesses (device)
    const S *Si, *hi, *hc, *aleph, *Tint, *Ei, *Es;
    S *Qio, *frazil, *Js, *Jw, *Tb, *Sb;
};

template <class S> struct InterpArgs {
    Layout2 L;
    nesf_exchange_coords coords;
    nesf_atmos_grid atmos;
    double tn;
    const S* src[9];          // u v T q p rain snow sw lw (atmosphere grid, 2 snapshots)
    S* dst[9];                // exchange-grid outputs
    const double *frac_i, *frac_j;
    // the tiled kernel (regular grids, no caches): exchange rows per tile and the largest
    // coarse footprint (columns x rows) a tile stages; 0: the per-cell gather kernel
    int tile_rows, fp_w, fp_h;
};

template <class S> struct AsmFields {
    const uint8_t* inactive;
    const S *aleph, *To, *rain, *snow, *isnow, *land_fw;
    const S *ao_QT, *ao_Qv, *ao_Jv, *ao_tx, *ao_ty, *ao_Ts;
    const S *io_Q, *io_Qf, *io_Js, *io_Jw, *io_tx, *io_ty;
    const S *ai_QT, *ai_Qv, *ai_tx, *ai_ty, *ai_Ts;
    const S *sw, *lw;
    S *o_u, *o_v, *o_T, *o_S, *o_eta, *o_H;
    S *i_top, *i_snow, *i_u, *i_v, *i_bottom;
    S *o_up_lw, *o_dn_lw, *o_dn_sw, *i_up_lw, *i_dn_lw, *i_dn_sw;
};

template <class S> struct AsmArgs {
    Layout2 L;
    int with_radiation;       // fuse apply_air_sea(_ice)_radiative_fluxes into the assembly
    AsmFields<S> f;
};

template <class S> struct LandArgs {
    Layout2 L;
    const uint8_t* inactive;
    const S *rain, *QT, *Qv, *Jv, *Ts, *sw, *lw;
    S *Es, *P, *E, *Jvo, *Pl;       // SlabLand accumulators
    S *up_lw, *dn_lw, *dn_sw;       // radiation diagnostics
};

// part 0: fluxes + frazil adjustment of T3; 1: the fluxes alone (T3 read only); 2: the adjustment alone.
template <class S> cudaError_t launch_io(const IOArgs<S>& a, const nesf_io_params& p, cudaStream_t s, int part = 0);
cudaError_t launch_frac(const Layout2& L, const nesf_exchange_coords& c, const nesf_atmos_grid& ag, double* fi,
                        double* fj, cudaStream_t s);
template <class S> cudaError_t launch_interp(const InterpArgs<S>& a, cudaStream_t s);
// Whether `fn` is one of the interpolation kernels of the storage type, to find its node
// in a captured graph.
bool is_interp_kernel(const void* fn, bool fp64);
// which: 0 net ocean, 1 net sea ice, 2 ocean radiation, 3 sea-ice radiation
template <class S>
cudaError_t launch_assemble(const AsmArgs<S>& a, const nesf_assembly_params& p, int which, cudaStream_t s);

// radiation false: the SlabLand accumulators; true: the radiative part added to surface_energy_flux
template <class S>
cudaError_t launch_land(const LandArgs<S>& a, const nesf_land_radiation_params& p, bool radiation, cudaStream_t s);

}  // namespace nesf
