"""The oracle's coupling step on a band of rows -- TEST INFRASTRUCTURE ONLY.

Used by tests/ and by bench.py's error statistics and CPU baseline as the checker
of the GPU step; the product path never calls it. It runs update_state!'s
interface-flux phases (time_step_earth_system_model.jl:50-80) with the C oracle on
the rows j = lo+1 .. lo+rows of a workload:

  1. interpolate_state! of the prescribed atmosphere onto the band
     (interpolate_atmospheric_state.jl:91-137), when the workload has one;
  2. the atmosphere-ocean solve (atmosphere_ocean_fluxes.jl:80-197);
  3. the atmosphere-sea-ice solve (atmosphere_sea_ice_fluxes.jl:65-185), when the
     workload has sea ice;
  4. the sea-ice-ocean fluxes with the frazil adjustment of the ocean temperature
     (sea_ice_ocean_fluxes.jl:106-226);
  5. the net ocean and sea-ice flux assembly with the radiative add-ons
     (assemble_net_ocean_fluxes.jl:74-153, assemble_net_sea_ice_fluxes.jl:42-81,
     apply_air_sea_radiative_fluxes.jl:62-111, apply_air_sea_ice_radiative_fluxes.jl:55-90).

Every phase is per cell (the assembly reads the west and south neighbours, the
face-centred ocean velocities the east and north ones), so a band of parent rows
[lo, lo + rows + 2 hy) with the workload's halos gives the same values on its
interior as the whole grid: the band's interior rows 1..rows are the workload's
rows lo+1..lo+rows. FP32 workloads are widened to FP64 (exact), so the oracle
computes the FP64 answer of the same inputs.
"""
import numpy as np

from nesf import api
from nesf import fields as F
from nesf import synthetic as syn

from . import oracle

ATMOS_TO_EXCHANGE = (("u", "u_atm"), ("v", "v_atm"), ("T", "T_atm"), ("q", "q_atm"), ("p", "p_atm"),
                     ("rain", "rain"), ("snow", "snow"), ("sw", "sw_down"), ("lw", "lw_down"))
OCEAN_NET = ("ocean_u", "ocean_v", "ocean_T", "ocean_S", "ocean_eta", "ocean_heat_content")
ICE_NET = ("ice_top_heat", "ice_top_snowfall", "ice_top_u", "ice_top_v", "ice_bottom_heat")
RAD_DIAG = ("ocean_upwelling_longwave", "ocean_downwelling_longwave", "ocean_downwelling_shortwave",
            "ice_upwelling_longwave", "ice_downwelling_longwave", "ice_downwelling_shortwave")


def band_rows(state, lo, rows):
    """The band's layout and the slice of parent rows it covers."""
    L = state.layout
    return syn.Layout(L.nx, rows, L.hx, L.hy), slice(lo, lo + rows + 2 * L.hy)


def band_of(array, state, lo, rows):
    """The band's parent rows of a full-grid parent array (FP64 copy; masks unchanged)."""
    _, rs = band_rows(state, lo, rows)
    a = np.asarray(array)[rs]
    return np.ascontiguousarray(a if a.dtype == np.uint8 else a.astype(np.float64))


def step_band(state, lo, rows, ao_spec, ai_spec=None, io_spec=None, asm_spec=None, time_weight=None,
              dz_top=10.0, atmos=None):
    """The oracle's coupling step on rows lo+1..lo+rows; returns (layout, results) with
    results = {"atmos": {...}, "ao": {...}, "ai": {...}, "io": {...}, "net": {...},
    "inputs": {...}} of band-sized FP64 parent arrays ("ao"/"ai" include "iterations";
    "inputs" holds the band's inputs, the interpolated atmosphere included).

    `atmos` (optional): the band's exchange-grid atmosphere (u_atm, ..., lw_down: band-sized
    parent arrays) to solve from instead of the oracle's own interpolation -- e.g. the
    values a GPU step with FP32 fields interpolated in FP32 arithmetic and then read, so
    that the solves are compared on the same inputs; "atmos" in the results is still the
    oracle's interpolation."""
    sub, _ = band_rows(state, lo, rows)
    band = {k: band_of(v, state, lo, rows) for k, v in state.fields.items() if v.ndim == 2}
    res = {"inputs": band}
    if state.atmos is not None:
        at = state.atmos
        c = state.coords
        bc = api.exchange_coords(syn.LonLat(c.lon0, c.dlon, c.lat0 + lo * c.dlat, c.dlat))
        tw = at["time_weight"] if time_weight is None else time_weight
        out = oracle.interpolate(sub, bc, api.atmos_grid_struct(at), at["arrays"], tw)
        res["atmos"] = {k: out[n] for n, k in ATMOS_TO_EXCHANGE}
        for n, k in ATMOS_TO_EXCHANGE:
            band[k] = out[n]
    if atmos is not None:
        for _, k in ATMOS_TO_EXCHANGE:
            if k in atmos:
                band[k] = np.ascontiguousarray(atmos[k], dtype=np.float64)
    res["ao"] = oracle.ao_fluxes(ao_spec.to_c(), sub, band)
    ice = ai_spec is not None and "ice_concentration" in band
    if ice:
        res["ai"] = oracle.ai_fluxes(ai_spec.to_c(), sub, band, band["ice_temperature"])
    if io_spec is not None and ice:
        plane = sub.shape[0] * sub.shape[1]
        io_in = {"ice_salinity": band["ice_salinity"], "ice_thickness": band["ice_thickness"],
                 "consolidation_thickness": band["consolidation_thickness"],
                 "ice_concentration": band["ice_concentration"], "internal_temperature": band["ice_temperature"],
                 "ice_mass_flux": band["ice_mass_flux"], "snow_mass_flux": band["snow_mass_flux"]}
        res["io"] = oracle.io_fluxes(io_spec.to_c(nz=1, stride_k=plane), sub, io_in, band["T_oc"][None],
                                     band["S_oc"][None], np.array([dz_top]))
    if asm_spec is not None and ice and "io" in res:
        ao, ai, io = res["ao"], res["ai"], res["io"]
        zero = np.zeros(sub.shape)
        arr = dict(inactive=band["inactive"], ice_concentration=band["ice_concentration"],
                   ocean_surface_temperature=np.ascontiguousarray(io["T_oc"][0]), rain=band["rain"],
                   snow=band["snow"], intercepted_snow=zero, ao_sensible=ao["sensible_heat"],
                   ao_latent=ao["latent_heat"], ao_water_vapor=ao["water_vapor"], ao_x_momentum=ao["x_momentum"],
                   ao_y_momentum=ao["y_momentum"], ao_interface_temperature=ao["interface_temperature"],
                   io_interface_heat=io["interface_heat"], io_frazil_heat=io["frazil_heat"], io_salt=io["salt"],
                   io_freshwater=io["freshwater"], io_x_momentum=zero, io_y_momentum=zero,
                   ai_sensible=ai["sensible_heat"], ai_latent=ai["latent_heat"], ai_x_momentum=ai["x_momentum"],
                   ai_y_momentum=ai["y_momentum"], ai_interface_temperature=ai["interface_temperature"],
                   sw_down=band["sw_down"], lw_down=band["lw_down"])
        net = {k: np.zeros(sub.shape) for k in OCEAN_NET + ICE_NET + RAD_DIAG}
        arr.update(net)
        pc = asm_spec.to_c()
        for which in ("ocean", "sea_ice", "ocean_radiation", "sea_ice_radiation"):
            oracle.assemble(pc, sub, arr, which)
        res["net"] = net
    return sub, res


def band_positions(state, rows, count):
    """`count` band starts spread evenly over the workload's rows."""
    L = state.layout
    return np.unique(np.linspace(0, L.ny - rows, count).astype(int))


def relative_errors(got, ref, floor):
    """|got - ref| / max(|ref|, floor) per cell (NaN in both: 0; in one: inf)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.maximum(np.abs(ref), floor)
    e = np.abs(got - ref) / np.where(den > 0, den, 1.0)
    e = np.where(np.isnan(got) & np.isnan(ref), 0.0, e)
    return np.where(np.isnan(got) ^ np.isnan(ref), np.inf, e)


class ErrorTable:
    """Max and 99th-percentile relative error per output over many bands. Each output's
    floor is 1e-6 of its largest oracle magnitude over all bands (cells where the flux
    nearly vanishes are compared on that absolute scale). "normwise" is the largest
    absolute error over the largest oracle magnitude: the measure for sums of terms that
    cancel (the net fluxes), whose per-cell relative error grows without bound where
    the sum vanishes."""

    def __init__(self):
        self.pairs = {}

    def add(self, name, got, ref, keep=None):
        g = np.asarray(got, np.float64).ravel()
        r = np.asarray(ref, np.float64).ravel()
        if keep is not None:
            k = np.asarray(keep).ravel()
            g, r = g[k], r[k]
        self.pairs.setdefault(name, []).append((g, r))

    def summary(self):
        out = {}
        for name, parts in self.pairs.items():
            g = np.concatenate([p[0] for p in parts])
            r = np.concatenate([p[1] for p in parts])
            finite = np.abs(r[np.isfinite(r)])
            floor = 1e-6 * finite.max() if finite.size else 0.0
            e = relative_errors(g, r, floor)
            ok = np.isfinite(g) & np.isfinite(r)
            norm = float(np.abs(g - r)[ok].max() / finite.max()) if ok.any() and finite.size and finite.max() > 0 \
                else 0.0
            out[name] = {"max": float(e.max()) if e.size else 0.0,
                         "p99": float(np.percentile(e, 99)) if e.size else 0.0,
                         "normwise": norm, "cells": int(e.size)}
        return out
