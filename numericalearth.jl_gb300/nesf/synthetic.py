"""Seeded synthetic surface states for the interface-flux workloads.

The reference drives this path with JRA55 / ECCO data; no dataset is available
here, so seeded fields with the stated distributions stand in for them. Every
array is an Oceananigans-style parent array: numpy shape (ny + 2hy, nx + 2hx),
C order, so i is fastest and element (i, j) (1-based interior index) lives at
[j - 1 + hy, i - 1 + hx]. Halos are filled periodically in longitude and by
copying the edge row in latitude, as Oceananigans' halo fill would for a
periodic-in-longitude, bounded-in-latitude grid.

Workloads (sizes are interior cells):
  ao_1deg          360 x 180 longitude-latitude, no land, one member, FP64,
                   atmosphere on the same grid;
  ao_quarter_land  1440 x 560 (lat -70..70) with a 30 % land mask from a
                   thresholded smoothed Gaussian field, atmosphere 640 x 320 at two
                   3-hourly snapshots interpolated in space and time, FP32;
  coupled_1440     1440 x 600 (lat -75..75) ocean + sea ice, sea ice poleward of
                   55 degrees, T_air - T_surface ~ N(0, 6) K, FP32;
  ensemble_32      32 members of 720 x 360 with perturbed bulk parameters, FP32;
  coupled_eighth   2880 x 1280 (lat -80..80) ocean + sea ice + 30 % land, atmosphere
                   640 x 320 x 2 snapshots interpolated onto the exchange grid, FP32.
"""
import math
from dataclasses import dataclass, field
from typing import Dict, Optional

import numpy as np

from .params import AtmosphereThermodynamicsParameters, celsius_to_kelvin

HALO = 3


def esat_liquid(T, th=None):
    """Saturation vapour pressure over liquid (Clausius-Clapeyron with linear L)."""
    th = th or AtmosphereThermodynamicsParameters()
    dcp = th.water_vapor_heat_capacity - th.liquid_water_heat_capacity
    Rv = th.R_v
    return th.triple_point_pressure * (T / th.triple_point_temperature) ** (dcp / Rv) * np.exp(
        (th.reference_vaporization_enthalpy - dcp * th.reference_temperature) / Rv *
        (1 / th.triple_point_temperature - 1 / T))


def specific_humidity_from_rh(RH, T, p, th=None):
    th = th or AtmosphereThermodynamicsParameters()
    e = RH * esat_liquid(T, th)
    einv = 1 / th.Rv_over_Rd
    return einv * e / (p - (1 - einv) * e)


def pad(interior, hx=HALO, hy=HALO):
    """Interior (ny, nx) -> parent array with periodic x halo and edge-copied y halo."""
    a = np.pad(interior, ((0, 0), (hx, hx)), mode="wrap")
    return np.pad(a, ((hy, hy), (0, 0)), mode="edge")


@dataclass
class Layout:
    nx: int
    ny: int
    hx: int = HALO
    hy: int = HALO

    @property
    def stride_j(self):
        return self.nx + 2 * self.hx

    @property
    def shape(self):
        return (self.ny + 2 * self.hy, self.nx + 2 * self.hx)

    def interior(self, a):
        return a[self.hy:self.hy + self.ny, self.hx:self.hx + self.nx]

    def ring(self, a):
        """Halo-ring launch range (0:nx+1, 0:ny+1)."""
        return a[self.hy - 1:self.hy + self.ny + 1, self.hx - 1:self.hx + self.nx + 1]


@dataclass
class LonLat:
    lon0: float
    dlon: float
    lat0: float
    dlat: float


def lonlat(nx, ny, lat_s, lat_n, lon_w=0.0, lon_e=360.0):
    dlon = (lon_e - lon_w) / nx
    dlat = (lat_n - lat_s) / ny
    return LonLat(lon_w + dlon / 2, dlon, lat_s + dlat / 2, dlat)


def centres(layout, c):
    """Longitude and latitude of every parent-array cell (halo included)."""
    i = np.arange(1 - layout.hx, layout.nx + layout.hx + 1)
    j = np.arange(1 - layout.hy, layout.ny + layout.hy + 1)
    lon = c.lon0 + (i - 1) * c.dlon
    lat = c.lat0 + (j - 1) * c.dlat
    return np.meshgrid(lon, lat)


def land_mask(rng, nx, ny, fraction=0.3, sigma=8.0):
    """Top `fraction` of a smoothed N(0,1) field (periodic in longitude)."""
    from scipy.ndimage import gaussian_filter
    g = rng.standard_normal((ny, nx))
    s = gaussian_filter(g, sigma=sigma, mode=("nearest", "wrap"))
    thresh = np.quantile(s, 1 - fraction)
    return (s > thresh).astype(np.uint8)


@dataclass
class SurfaceState:
    """Exchange-grid state of one workload, as host numpy arrays."""
    layout: Layout
    coords: LonLat
    dtype: type
    fields: Dict[str, np.ndarray] = field(default_factory=dict)
    atmos: Optional[dict] = None          # coarse prescribed atmosphere (interpolated workloads)
    members: int = 1

    def __getitem__(self, k):
        return self.fields[k]


def _ocean_interior(rng, lat, nx, ny):
    coslat = np.cos(np.deg2rad(lat))
    sst = 271 + 32 * coslat ** 2 + rng.normal(0, 0.5, (ny, nx))
    S = rng.uniform(30, 38, (ny, nx))
    uo = rng.normal(0, 0.3, (ny, nx))
    vo = rng.normal(0, 0.3, (ny, nx))
    return sst, S, uo, vo


def _atmos_interior(rng, surface_T, nx, ny, dT_mean=-1.0, dT_std=2.0):
    """10 m wind ~ N(0, 7), T_air = surface_T + N(dT_mean, dT_std), RH ~ U(0.6, 0.95),
    p ~ 101325 + N(0, 1000), SW ~ U(0, 1000), LW ~ U(300, 450)."""
    ua = rng.normal(0, 7, (ny, nx))
    va = rng.normal(0, 7, (ny, nx))
    Ta = surface_T + rng.normal(dT_mean, dT_std, (ny, nx))
    RH = rng.uniform(0.6, 0.95, (ny, nx))
    p = 101325 + rng.normal(0, 1000, (ny, nx))
    qa = specific_humidity_from_rh(RH, Ta, p)
    sw = rng.uniform(0, 1000, (ny, nx))
    lw = rng.uniform(300, 450, (ny, nx))
    return dict(u=ua, v=va, T=Ta, q=qa, p=p, sw=sw, lw=lw)


def ao_1deg(seed=1000, nx=360, ny=180, dtype=np.float64, halo=HALO):
    """Atmosphere-ocean, 1 degree, no land, atmosphere on the exchange grid."""
    rng = np.random.default_rng(seed)
    L = Layout(nx, ny, halo, halo)
    c = lonlat(nx, ny, -90.0, 90.0)
    _, lat = centres(L, c)
    lat_int = L.interior(lat)
    sst, S, uo, vo = _ocean_interior(rng, lat_int, nx, ny)
    at = _atmos_interior(rng, sst, nx, ny)
    f = {
        "u_atm": at["u"], "v_atm": at["v"], "T_atm": at["T"], "p_atm": at["p"], "q_atm": at["q"],
        "sw_down": at["sw"], "lw_down": at["lw"],
        "u_oc": uo, "v_oc": vo, "T_oc": sst - celsius_to_kelvin, "S_oc": S,
    }
    st = SurfaceState(L, c, dtype)
    st.fields = {k: pad(v, halo, halo).astype(dtype) for k, v in f.items()}
    st.fields["inactive"] = np.zeros(L.shape, np.uint8)
    return st


def al_1deg(seed=1100, nx=360, ny=180, dtype=np.float64, halo=HALO, dry_fraction=0.2):
    """Atmosphere-land, 1 degree, all land, atmosphere on the exchange grid: bulk land
    temperature 271 + 32 cos^2(lat) + N(0, 3) K (kelvin), surface saturation U(0, 1) with
    `dry_fraction` of the cells dry (0), the atmosphere as over the ocean."""
    rng = np.random.default_rng(seed)
    L = Layout(nx, ny, halo, halo)
    c = lonlat(nx, ny, -90.0, 90.0)
    _, lat = centres(L, c)
    lat_int = L.interior(lat)
    T = 271 + 32 * np.cos(np.deg2rad(lat_int)) ** 2 + rng.normal(0, 3, (ny, nx))
    at = _atmos_interior(rng, T, nx, ny)
    sat = rng.uniform(0, 1, (ny, nx))
    sat[rng.uniform(0, 1, (ny, nx)) < dry_fraction] = 0.0
    f = {"u_atm": at["u"], "v_atm": at["v"], "T_atm": at["T"], "p_atm": at["p"], "q_atm": at["q"],
         "land_temperature": T, "saturation": sat}
    st = SurfaceState(L, c, dtype)
    st.fields = {k: pad(v, halo, halo).astype(dtype) for k, v in f.items()}
    return st


def _coarse_atmosphere(rng, nxa=640, nya=320, halo=HALO, dtype=np.float32, nt=2, dT_mean=-1.0, dT_std=2.0):
    """Global prescribed atmosphere (JRA55-like 0.5625 degree) with nt snapshots 3 h apart.
    Air temperature follows 271 + 32 cos^2(lat), cooled by up to 30 K poleward of 50 degrees."""
    La = Layout(nxa, nya, halo, halo)
    ca = lonlat(nxa, nya, -90.0, 90.0)
    _, lat = centres(La, ca)
    lat_int = La.interior(lat)
    base = 271 + 32 * np.cos(np.deg2rad(lat_int)) ** 2 - 30 * np.clip((np.abs(lat_int) - 50) / 40, 0, 1)
    snaps = {k: [] for k in ("u", "v", "T", "q", "p", "rain", "snow", "sw", "lw")}
    for _ in range(nt):
        at = _atmos_interior(rng, base, nxa, nya, dT_mean, dT_std)
        at["rain"] = rng.exponential(2e-5, (nya, nxa))     # kg m^-2 s^-1
        at["snow"] = rng.exponential(5e-6, (nya, nxa))
        for k in snaps:
            snaps[k].append(pad(at[k], halo, halo).astype(dtype))
    arrays = {k: np.ascontiguousarray(np.stack(v)) for k, v in snaps.items()}
    return dict(layout=La, coords=ca, arrays=arrays, stride_t=La.shape[0] * La.shape[1], time_weight=1.0 / 3.0)


def _sea_ice(rng, lat_int, sst, nx, ny, lat_ice=55.0):
    ice = np.abs(lat_int) > lat_ice
    aleph = np.where(ice, rng.uniform(0, 1, (ny, nx)), 0.0)
    hi = rng.uniform(0, 3, (ny, nx))
    hs = rng.uniform(0, 0.5, (ny, nx))
    Tice = rng.uniform(240, 273, (ny, nx))
    Si = np.full((ny, nx), 4.0)           # sea_ice_simulation ice_salinity = 4
    hc = np.full((ny, nx), 0.05)          # ice_consolidation_thickness = 0.05
    Ei = rng.normal(0, 1e-4, (ny, nx)) * ice
    Es = rng.normal(0, 2e-5, (ny, nx)) * ice
    return dict(ice_concentration=aleph, ice_thickness=hi, snow_thickness=hs,
                ice_temperature=Tice - celsius_to_kelvin, ice_salinity=Si, consolidation_thickness=hc,
                ice_mass_flux=Ei, snow_mass_flux=Es)


def coupled(seed=1004, nx=2880, ny=1280, lat_s=-80.0, lat_n=80.0, land=0.3, interpolate=True,
            dtype=np.float32, halo=HALO, dT_std=6.0):
    """Ocean + sea ice (+ land) on a longitude-latitude exchange grid, atmosphere either
    prescribed on a 640 x 320 grid (interpolate=True) or given on the exchange grid."""
    rng = np.random.default_rng(seed)
    L = Layout(nx, ny, halo, halo)
    c = lonlat(nx, ny, lat_s, lat_n)
    _, lat = centres(L, c)
    lat_int = L.interior(lat)
    sst, S, uo, vo = _ocean_interior(rng, lat_int, nx, ny)
    ice = _sea_ice(rng, lat_int, sst, nx, ny)
    # Ocean under sea ice sits near its freezing point; a few cells are supercooled (frazil)
    Tf = -0.054 * S + celsius_to_kelvin
    sst = np.where(ice["ice_concentration"] > 0, Tf + rng.uniform(-0.05, 0.5, (ny, nx)), sst)
    mask = land_mask(rng, nx, ny, land) if land > 0 else np.zeros((ny, nx), np.uint8)
    f = {"u_oc": uo, "v_oc": vo, "T_oc": sst - celsius_to_kelvin, "S_oc": S}
    f.update(ice)
    st = SurfaceState(L, c, dtype)
    if interpolate:
        st.atmos = _coarse_atmosphere(rng, dtype=dtype, halo=halo, dT_mean=0.0, dT_std=dT_std)
    else:
        # Surface temperature the air is relative to: ice where concentrated, else SST
        Tsurf = np.where(ice["ice_concentration"] > 0.5, ice["ice_temperature"] + celsius_to_kelvin, sst)
        at = _atmos_interior(rng, Tsurf, nx, ny, 0.0, dT_std)
        at["rain"] = rng.exponential(2e-5, (ny, nx))
        at["snow"] = rng.exponential(5e-6, (ny, nx))
        f.update({"u_atm": at["u"], "v_atm": at["v"], "T_atm": at["T"], "p_atm": at["p"], "q_atm": at["q"],
                  "sw_down": at["sw"], "lw_down": at["lw"], "rain": at["rain"], "snow": at["snow"]})
    st.fields = {k: pad(v, halo, halo).astype(dtype) for k, v in f.items()}
    st.fields["inactive"] = pad(mask, halo, halo)
    return st


def warm_training_state(seed, nx=720, ny=360, dtype=np.float32, halo=HALO):
    """Training states of the warm-start network: open ocean (no land, no ice) from 80 S to
    80 N with the atmosphere on the exchange grid, the 1-degree distributions widened to
    10 m wind speeds U(0, 40) m/s in a uniform direction and air - sea temperature
    differences U(-15, +10) K."""
    rng = np.random.default_rng(seed)
    L = Layout(nx, ny, halo, halo)
    c = lonlat(nx, ny, -80.0, 80.0)
    _, lat = centres(L, c)
    lat_int = L.interior(lat)
    sst, S, uo, vo = _ocean_interior(rng, lat_int, nx, ny)
    at = _atmos_interior(rng, sst, nx, ny)
    speed = rng.uniform(0.0, 40.0, (ny, nx))
    angle = rng.uniform(0.0, 2 * np.pi, (ny, nx))
    at["u"], at["v"] = speed * np.cos(angle), speed * np.sin(angle)
    at["T"] = sst + rng.uniform(-15.0, 10.0, (ny, nx))
    RH = rng.uniform(0.6, 0.95, (ny, nx))
    at["q"] = specific_humidity_from_rh(RH, at["T"], at["p"])
    f = {"u_atm": at["u"], "v_atm": at["v"], "T_atm": at["T"], "p_atm": at["p"], "q_atm": at["q"],
         "sw_down": at["sw"], "lw_down": at["lw"], "u_oc": uo, "v_oc": vo, "T_oc": sst - celsius_to_kelvin,
         "S_oc": S}
    st = SurfaceState(L, c, dtype)
    st.fields = {k: pad(v, halo, halo).astype(dtype) for k, v in f.items()}
    st.fields["inactive"] = np.zeros(L.shape, np.uint8)
    return st


def ao_quarter_land(seed=1001, **kw):
    kw.setdefault("nx", 1440)
    kw.setdefault("ny", 560)
    return coupled(seed=seed, lat_s=-70.0, lat_n=70.0, land=0.3, interpolate=True, **kw)


def coupled_1440(seed=1002, **kw):
    kw.setdefault("nx", 1440)
    kw.setdefault("ny", 600)
    return coupled(seed=seed, lat_s=-75.0, lat_n=75.0, land=0.0, interpolate=False, **kw)


def coupled_eighth(seed=1004, **kw):
    kw.setdefault("nx", 2880)
    kw.setdefault("ny", 1280)
    return coupled(seed=seed, lat_s=-80.0, lat_n=80.0, land=0.3, interpolate=True, **kw)


def ensemble_params(seed, members):
    """Per-member perturbations: Charnock U(0.008, 0.02), gustiness velocity U(0.2, 1.0)
    as minimum_gustiness, scalar-roughness A, b and smooth-wall parameter x U(0.8, 1.2)."""
    rng = np.random.default_rng(seed * 100)
    return [dict(charnock=rng.uniform(0.008, 0.02), minimum_gustiness=rng.uniform(0.2, 1.0),
                 A_scale=rng.uniform(0.8, 1.2), b_scale=rng.uniform(0.8, 1.2),
                 nu_scale=rng.uniform(0.8, 1.2)) for _ in range(members)]


def ensemble_member_spec(pert):
    """The atmosphere-ocean interface of one ensemble member: SimilarityTheoryFluxes with the
    member's Charnock parameter, minimum gustiness, smooth-wall parameter (0.11 scaled) and
    Reynolds-scaling A, b (5.85e-5, 0.72 scaled) for both scalar roughness lengths."""
    from . import params as P
    mom = P.MomentumRoughnessLength(wave_formulation=pert["charnock"],
                                    smooth_wall_parameter=0.11 * pert["nu_scale"])
    sc = P.ScalarRoughnessLength(reynolds_number_scaling_function=P.ReynoldsScalingFunction(
        5.85e-5 * pert["A_scale"], 0.72 * pert["b_scale"]))
    flux = P.SimilarityTheoryFluxes(subgrid_velocities=P.ConvectiveGustiness(1.2, pert["minimum_gustiness"]),
                                    momentum_roughness_length=mom, temperature_roughness_length=sc,
                                    water_vapor_roughness_length=sc)
    return P.atmosphere_ocean_interface_spec(flux_formulation=flux)


def ensemble(seed=1003, members=32, nx=720, ny=360, dtype=np.float32, halo=HALO):
    """`members` AO problems back to back (member stride = one parent array)."""
    states = [ao_1deg(seed * 100 + m, nx, ny, dtype, halo) for m in range(members)]
    st = SurfaceState(states[0].layout, states[0].coords, dtype, members=members)
    st.fields = {k: np.ascontiguousarray(np.stack([s.fields[k] for s in states])) for k in states[0].fields}
    st.perturbations = ensemble_params(seed, members)
    return st
