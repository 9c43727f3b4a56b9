"""ctypes front end of the CPU oracle (oracle/nesf_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker. The product path never calls it.
Inputs are numpy arrays; FP32 workloads are widened to FP64 before the call
(every FP32 value is exact in FP64), so the oracle always computes in FP64.
"""
import contextlib
import ctypes as C
import os
import sys

import numpy as np

_REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_PKG = os.path.join(_REPO, "numericalearth.jl_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from nesf import _abi as A            # noqa: E402
from nesf import fields as F          # noqa: E402

from . import build as _build          # noqa: E402

_LIB = None
P = C.POINTER
vp = C.c_void_p
d = C.c_double


def load():
    global _LIB
    if _LIB is None:
        lib = C.CDLL(_build.build())
        sig = {
            "oracle_saturation_vapor_pressure": (d, [P(A.ThermodynamicsParameters), d, C.c_int32]),
            "oracle_air_density": (d, [P(A.ThermodynamicsParameters), d, d, d]),
            "oracle_cp_m": (d, [P(A.ThermodynamicsParameters), d]),
            "oracle_latent_heat_vapor": (d, [P(A.ThermodynamicsParameters), d]),
            "oracle_latent_heat_sublim": (d, [P(A.ThermodynamicsParameters), d]),
            "oracle_virtual_temperature": (d, [P(A.ThermodynamicsParameters), d, d]),
            "oracle_surface_specific_humidity": (d, [P(A.InterfaceParams), d, d]),
            "oracle_dry_layer_humidity": (d, [P(A.InterfaceParams)] + [d] * 9),
            "oracle_pow_ten_thirds": (d, [d]),
            "oracle_stability": (d, [P(A.StabilityFunction), d]),
            "oracle_neutral_drag": (d, [P(A.CoefficientFluxes), d]),
            "oracle_al_fluxes": (C.c_int, [P(A.InterfaceParams), P(A.ALFields)]),
            "oracle_vsgs2": (d, [P(A.SimilarityTheoryFluxesC), d, d, d]),
            "oracle_momentum_roughness": (d, [P(A.RoughnessLength), d, d, d]),
            "oracle_scalar_roughness": (d, [P(A.RoughnessLength), d, d, d, d]),
            "oracle_buoyancy_scale": (d, [P(A.InterfaceParams), d, d, d, d]),
            "oracle_solve_interface_conditions": (None, [P(A.IOParams), d, d, d, d, d, d, P(d), P(d), P(d)]),
            "oracle_ao_fluxes": (C.c_int, [P(A.InterfaceParams), P(A.AOFields)]),
            "oracle_ai_fluxes": (C.c_int, [P(A.InterfaceParams), P(A.AIFields)]),
            "oracle_io_fluxes": (C.c_int, [P(A.IOParams), P(A.IOFields)]),
            "oracle_fractional_indices": (C.c_int, [P(A.Grid), P(A.ExchangeCoords), P(A.AtmosGrid), vp, vp]),
            "oracle_interpolate_atmosphere": (C.c_int, [P(A.InterpFields)]),
            "oracle_assemble_net_ocean_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields)]),
            "oracle_assemble_net_sea_ice_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields)]),
            "oracle_apply_air_sea_radiative_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields)]),
            "oracle_apply_air_sea_ice_radiative_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields)]),
            "oracle_assemble_net_land_fluxes": (C.c_int, [P(A.LandFluxFields)]),
            "oracle_apply_air_land_radiative_fluxes": (C.c_int, [P(A.LandRadiationParams), P(A.LandFluxFields)]),
            "oracle_set_threads": (None, [C.c_int32]),
            "oracle_set_humidity_ulp_shift": (None, [C.c_int32, C.c_int32]),
            "oracle_set_temperature_ulp_shift": (None, [C.c_int32]),
            "oracle_set_interface_temperature_ulp_shift": (None, [C.c_int32]),
            "oracle_get_threads": (C.c_int32, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def _f64(a):
    if a is None:
        return None
    if a.dtype == np.uint8 or a.dtype == np.int32:
        return np.ascontiguousarray(a)
    return np.ascontiguousarray(a, dtype=np.float64)


def _check(code, what):
    if code != 0:
        raise RuntimeError(f"{what} returned {code}")


def ao_fluxes(params, layout, inputs, with_iterations=True):
    """Run the AO solve on host arrays; returns a dict of FP64 outputs (+ 'iterations')."""
    lib = load()
    shape = layout.shape
    outs = {k: np.zeros(shape) for k in F.AO_OUTPUTS}
    arrays = {k: _f64(inputs.get(k)) for k in F.AO_INPUTS}
    arrays.update(outs)
    it = np.zeros(shape, np.int32) if with_iterations else None
    arrays["iterations"] = it
    f = F.pack(A.AOFields, F.make_grid(layout), arrays, dtype=A.NESF_F64)
    _check(lib.oracle_ao_fluxes(C.byref(params), C.byref(f)), "oracle_ao_fluxes")
    if with_iterations:
        outs["iterations"] = it
    return outs


def al_fluxes(params, layout, inputs, with_iterations=True):
    """oracle_al_fluxes on FP64 host arrays; returns the outputs (and iterations)."""
    lib = load()
    arrays = {k: _f64(inputs[k]) if inputs.get(k) is not None else None for k in F.AL_INPUTS}
    out = {k: np.zeros(layout.shape) for k in F.AL_OUTPUTS}
    arrays.update(out)
    its = np.zeros(layout.shape, dtype=np.int32) if with_iterations else None
    arrays["iterations"] = its
    f = F.pack(A.ALFields, F.make_grid(layout), arrays, dtype=A.NESF_F64)
    _check(lib.oracle_al_fluxes(C.byref(params), C.byref(f)), "oracle_al_fluxes")
    if with_iterations:
        out["iterations"] = its
    return out


@contextlib.contextmanager
def humidity_ulp_shift(n, carry):
    """Within the block every iterate's interface humidity is moved n units in the last place
    where its flux evaluation sees it, and with carry also in the iterate handed on
    (oracle_set_humidity_ulp_shift): the conditioning probe of the parity tests."""
    lib = load()
    lib.oracle_set_humidity_ulp_shift(n, 1 if carry else 0)
    try:
        yield
    finally:
        lib.oracle_set_humidity_ulp_shift(0, 0)


@contextlib.contextmanager
def temperature_ulp_shift(n, interface=False):
    """Within the block every iterate's air potential temperature theta_a (or, with interface,
    its interface temperature T_s) is moved n units in the last place
    (oracle_set_temperature_ulp_shift / oracle_set_interface_temperature_ulp_shift): the
    temperature side of the probe."""
    lib = load()
    setter = lib.oracle_set_interface_temperature_ulp_shift if interface else lib.oracle_set_temperature_ulp_shift
    setter(n)
    try:
        yield
    finally:
        setter(0)


def conditioning_response(run, ref, keys, shift=1024, view=None):
    """Per-cell response of the oracle's outputs to one unit in the last place of its interface
    humidity (with and without carrying the change into the next iterate), of theta_a and of
    the interface temperature T_s: the largest relative change over the four probes, each
    under a `shift`-ulp move, divided by `shift` (a single ulp rounds away in some cells).
    `run()` returns the oracle's outputs; `view(key, array)` selects the cells compared
    (default: all)."""
    view = view or (lambda k, a: a)
    outs = []
    for carry in (False, True):
        with humidity_ulp_shift(shift, carry):
            outs.append(run())
    for interface in (False, True):
        with temperature_ulp_shift(shift, interface):
            outs.append(run())
    resp = {}
    for k in keys:
        r = np.asarray(view(k, ref[k]), np.float64)
        scale = np.abs(r)
        finite = scale[np.isfinite(scale)]
        den = np.maximum(scale, 1e-6 * finite.max() if finite.size else 0.0)
        den = np.where(den > 0, den, 1.0)
        resp[k] = np.max([np.abs(np.asarray(view(k, o[k]), np.float64) - r) / den for o in outs], axis=0) / shift
    return resp


def ai_fluxes(params, layout, inputs, interface_temperature, with_iterations=True):
    lib = load()
    shape = layout.shape
    outs = {k: np.zeros(shape) for k in F.AI_OUTPUTS}
    Ts = np.array(interface_temperature, dtype=np.float64, copy=True)
    arrays = {k: _f64(inputs.get(k)) for k in F.AI_INPUTS}
    arrays.update(outs)
    arrays["interface_temperature"] = Ts
    it = np.zeros(shape, np.int32) if with_iterations else None
    arrays["iterations"] = it
    f = F.pack(A.AIFields, F.make_grid(layout), arrays, dtype=A.NESF_F64)
    _check(lib.oracle_ai_fluxes(C.byref(params), C.byref(f)), "oracle_ai_fluxes")
    outs["interface_temperature"] = Ts
    if with_iterations:
        outs["iterations"] = it
    return outs


def io_fluxes(params, layout, inputs, T3, S3, dz):
    """inputs: 2-D arrays; T3/S3: (nz, ny+2hy, nx+2hx) arrays; T3 is copied and returned mutated."""
    lib = load()
    shape = layout.shape
    T = np.array(T3, dtype=np.float64, copy=True)
    S = np.ascontiguousarray(S3, dtype=np.float64)
    dzv = np.ascontiguousarray(dz, dtype=np.float64)
    outs = {k: np.zeros(shape) for k in F.IO_OUTPUTS}
    arrays = {k: _f64(inputs.get(k)) for k in ("ice_salinity", "ice_thickness", "consolidation_thickness",
                                                "ice_concentration", "internal_temperature", "ice_mass_flux",
                                                "snow_mass_flux")}
    arrays.update(outs)
    arrays.update(T_oc=T, S_oc=S, dz=dzv)
    f = F.pack(A.IOFields, F.make_grid(layout), arrays, dtype=A.NESF_F64)
    _check(lib.oracle_io_fluxes(C.byref(params), C.byref(f)), "oracle_io_fluxes")
    outs["T_oc"] = T
    return outs


def interpolate(layout, coords, atmos_grid, atmos_arrays, time_weight, names=None):
    """atmos_arrays: dict u v T q p rain snow sw lw -> (2, nya+2h, nxa+2h) arrays."""
    lib = load()
    shape = layout.shape
    key = {"u": "u", "v": "v", "T": "T", "q": "q", "p": "p", "rain": "rain", "snow": "snow",
           "sw": "sw_down", "lw": "lw_down"}
    outname = {"u": "u_out", "v": "v_out", "T": "T_out", "q": "q_out", "p": "p_out", "rain": "rain_out",
               "snow": "snow_out", "sw": "sw_out", "lw": "lw_out"}
    names = names or list(key)
    arrays = {}
    outs = {}
    for n in names:
        arrays[key[n]] = _f64(atmos_arrays[n])
        outs[n] = np.zeros(shape)
        arrays[outname[n]] = outs[n]
    f = F.pack(A.InterpFields, F.make_grid(layout), arrays, dtype=A.NESF_F64,
               coords=coords, atmos=atmos_grid, time_weight=time_weight)
    _check(lib.oracle_interpolate_atmosphere(C.byref(f)), "oracle_interpolate_atmosphere")
    return outs


def assemble(params, layout, arrays, which):
    """which: 'ocean' | 'sea_ice' | 'ocean_radiation' | 'sea_ice_radiation'. Output arrays in
    `arrays` are updated in place (they must be float64 numpy arrays)."""
    lib = load()
    arrs = {k: (_f64(v) if not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags["C_CONTIGUOUS"])
                else v) for k, v in arrays.items()}
    f = F.pack(A.AssemblyFields, F.make_grid(layout), arrs, dtype=A.NESF_F64)
    fn = {"ocean": lib.oracle_assemble_net_ocean_fluxes, "sea_ice": lib.oracle_assemble_net_sea_ice_fluxes,
          "ocean_radiation": lib.oracle_apply_air_sea_radiative_fluxes,
          "sea_ice_radiation": lib.oracle_apply_air_sea_ice_radiative_fluxes}[which]
    _check(fn(C.byref(params), C.byref(f)), "oracle assembly")
    return arrs


def land_assembly(layout, arrays, radiation=None):
    """oracle_assemble_net_land_fluxes (radiation None) or oracle_apply_air_land_radiative_fluxes
    (radiation an nesf_land_radiation_params). Output arrays in `arrays` are updated in place
    (they must be float64 numpy arrays)."""
    lib = load()
    arrs = {k: (_f64(v) if not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags["C_CONTIGUOUS"])
                else v) for k, v in arrays.items()}
    f = F.pack(A.LandFluxFields, F.make_grid(layout), arrs, dtype=A.NESF_F64)
    if radiation is None:
        _check(lib.oracle_assemble_net_land_fluxes(C.byref(f)), "oracle_assemble_net_land_fluxes")
    else:
        _check(lib.oracle_apply_air_land_radiative_fluxes(C.byref(radiation), C.byref(f)),
               "oracle_apply_air_land_radiative_fluxes")
    return arrs


def set_threads(n):
    load().oracle_set_threads(int(n))


def get_threads():
    return int(load().oracle_get_threads())


def area_integrals(layout, fields, factors=None, inactive=None, area=None, row_area=None, uniform_area=1.0):
    """Exact area integrals (fractions.Fraction) of the interior cells, the checker of
    nesf_area_integrals: int dA(a) = sum(a) * A_z and int dA(a, b) = sum(a .* b) * A_z
    (test/test_conservation.jl:100-101). Cell terms are the FP64 products a * b * area
    rounded as the device rounds them; their sum is exact."""
    from fractions import Fraction
    I = layout.interior
    mask = np.ones((layout.ny, layout.nx), bool) if inactive is None else I(inactive) == 0
    factors = factors or [None] * len(fields)
    out = []
    for a, b in zip(fields, factors):
        x = I(np.asarray(a)).astype(np.float64)
        if b is not None:
            x = x * I(np.asarray(b)).astype(np.float64)
        if area is not None:
            x = x * I(np.asarray(area, dtype=np.float64))
        elif row_area is not None:
            x = x * np.asarray(row_area, dtype=np.float64)[:, None]
        terms = x[mask]
        total = sum((Fraction(float(t)) for t in terms), Fraction(0))
        if area is None and row_area is None:
            total *= Fraction(float(uniform_area))
        out.append(total)
    return out


def time_indices(times, indexing, period, t):
    """The bracketing snapshots (0-based n1, n2) of time t and the weight of n2, restated from
    the time indexing of Oceananigans' FieldTimeSeries (Cyclical / Linear / Clamp), which
    NumericalEarth's atmosphere interpolation calls (interpolate_atmospheric_state.jl:57-60;
    the package is not vendored with the reference, so this follows its documented behaviour:
    Cyclical wraps t into [t_0, t_0 + period) and blends the last snapshot into the first past
    t_last, its default period being the span plus the last interval; Linear extrapolates the
    end intervals; Clamp holds the end snapshots)."""
    times = np.asarray(times, dtype=np.float64)
    nt = len(times)
    if nt == 1:
        return 0, 0, 0.0
    t0, tl = float(times[0]), float(times[-1])
    if indexing == "cyclical":
        P = period if period and period > 0 else (tl - t0) + (tl - float(times[-2]))
        t = t0 + float(np.mod(t - t0, P))
        if t >= tl:
            return nt - 1, 0, (t - tl) / (t0 + P - tl)
    elif indexing == "clamp":
        if t <= t0:
            return 0, 0, 0.0
        if t >= tl:
            return nt - 1, nt - 1, 0.0
    n = int(np.searchsorted(times, t, side="right")) - 1
    n = min(max(n, 0), nt - 2)
    return n, n + 1, (t - float(times[n])) / (float(times[n + 1]) - float(times[n]))
