"""Host API: the reference's interface-flux entry points over libnesf.so.

Names follow NumericalEarth.jl (`compute_atmosphere_ocean_fluxes!` becomes
`compute_atmosphere_ocean_fluxes`, `update_state!` becomes `update_state`).
Arrays are torch CUDA tensors in the Oceananigans parent layout; torch only
provides device memory and streams, all arithmetic runs in libnesf.so.
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, Optional

import numpy as np

from . import _abi as A
from . import fields as F
from . import params as P
from ._lib import check, load

PRECISIONS = {"f64": A.PLAIN_F64, "plain": A.PLAIN_F64, "f32": A.F32_POLISH, "f32_polish": A.F32_POLISH,
              "f32_adaptive": A.F32_ADAPTIVE}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("nesf needs a CUDA device: there is no CPU path")
    return torch


def _stream_handle(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class Context:
    """Library-owned scratch (statistics, ensemble parameters) for one device."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.nesf_context_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.nesf_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_DEFAULT_CTX = {}


def default_context(device=None):
    torch = _torch()
    dev = torch.cuda.current_device() if device is None else device
    if dev not in _DEFAULT_CTX:
        _DEFAULT_CTX[dev] = Context(dev)
    return _DEFAULT_CTX[dev]


def solver_options(precision="f64", polish_maxiter=0, mlp=None, calm_replay_wind=None):
    """nesf_solver_options; `mlp` (a warm.WarmStartNetwork) turns on the learned warm start;
    `calm_replay_wind` (m/s) overrides the library's default for the sea-ice solve's calm cells.
    Launch shapes are the context's tuning (set_tuning, autotune), not options of a call."""
    o = A.SolverOptions()
    load().nesf_default_solver_options(C.byref(o))
    o.precision = PRECISIONS[precision]
    o.polish_maxiter = polish_maxiter
    if calm_replay_wind is not None:
        o.calm_replay_wind = float(calm_replay_wind)
    if mlp is not None:
        o.warm_start = 1
        o.mlp = mlp.ptr
    return o


def stats_dict(s):
    return {"cells": s.cells, "solved": s.solved, "iterations": s.iterations, "max_iterations": s.max_iterations,
            "nonconverged": s.nonconverged, "polished": s.polished, "polish_iterations": s.polish_iterations,
            "cold_fallbacks": s.cold_fallbacks, "fp64_redo": s.fp64_redo, "replay_reasons": list(s.replay_reasons), "histogram": np.array(s.histogram[:], dtype=np.int64)}


def _grid_of(layout):
    return F.make_grid(layout)


def compute_atmosphere_ocean_fluxes(spec, layout, state, out, precision="f64", polish_maxiter=0, stats=False,
                                    iterations=None, ctx=None, stream=None, mlp=None):
    """atmosphere_ocean_fluxes.jl:17-60 on device tensors. `state` holds AO inputs
    (fields.AO_INPUTS), `out` the AtmosphereSurfaceFluxes + interface temperature."""
    lib = load()
    arrays = {k: state.get(k) for k in F.AO_INPUTS}
    arrays.update({k: out.get(k) for k in F.AO_OUTPUTS})
    arrays["iterations"] = iterations
    f = F.pack(A.AOFields, _grid_of(layout), arrays)
    p = spec.to_c() if hasattr(spec, "to_c") else spec
    o = solver_options(precision, polish_maxiter, mlp=mlp)
    st = A.Stats() if stats else None
    ctx = ctx or default_context()
    check(lib.nesf_compute_atmosphere_ocean_fluxes(ctx.handle, C.byref(p), C.byref(f), C.byref(o),
                                                   C.byref(st) if st is not None else None, _stream_handle(stream)))
    return stats_dict(st) if st is not None else None


def compute_atmosphere_ocean_fluxes_ensemble(specs, layout, state, out, precision="f32", polish_maxiter=0,
                                             stats=False, iterations=None, ctx=None, stream=None):
    """Members stacked along the first tensor dimension, each with its own parameters."""
    lib = load()
    members = len(specs)
    arrays = {k: state.get(k) for k in F.AO_INPUTS}
    arrays.update({k: out.get(k) for k in F.AO_OUTPUTS})
    arrays["iterations"] = iterations
    f = F.pack(A.AOFields, _grid_of(layout), arrays)
    ps = (A.InterfaceParams * members)(*[s.to_c() if hasattr(s, "to_c") else s for s in specs])
    stride = layout.shape[0] * layout.shape[1]
    o = solver_options(precision, polish_maxiter)
    st = A.Stats() if stats else None
    ctx = ctx or default_context()
    check(lib.nesf_compute_atmosphere_ocean_fluxes_ensemble(ctx.handle, ps, members, stride, C.byref(f), C.byref(o),
                                                            C.byref(st) if st is not None else None,
                                                            _stream_handle(stream)))
    return stats_dict(st) if st is not None else None


def compute_atmosphere_sea_ice_fluxes(spec, layout, state, out, precision="f64", polish_maxiter=0, stats=False,
                                      iterations=None, ctx=None, stream=None, mlp=None, calm_replay_wind=None):
    """atmosphere_sea_ice_fluxes.jl:18-62; `out['interface_temperature']` is read as the
    initial skin temperature and overwritten with the solved one."""
    lib = load()
    arrays = {k: state.get(k) for k in F.AI_INPUTS}
    arrays.update({k: out.get(k) for k in F.AI_OUTPUTS})
    arrays["interface_temperature"] = out["interface_temperature"]
    arrays["iterations"] = iterations
    f = F.pack(A.AIFields, _grid_of(layout), arrays)
    p = spec.to_c() if hasattr(spec, "to_c") else spec
    o = solver_options(precision, polish_maxiter, mlp=mlp, calm_replay_wind=calm_replay_wind)
    st = A.Stats() if stats else None
    ctx = ctx or default_context()
    check(lib.nesf_compute_atmosphere_sea_ice_fluxes(ctx.handle, C.byref(p), C.byref(f), C.byref(o),
                                                     C.byref(st) if st is not None else None, _stream_handle(stream)))
    return stats_dict(st) if st is not None else None


def compute_atmosphere_land_fluxes(spec, layout, state, out, precision="f64", stats=False, iterations=None,
                                   ctx=None, stream=None):
    """atmosphere_land_fluxes.jl:48-105: `state` holds the exchange-grid atmosphere
    (u_atm, v_atm, T_atm, p_atm, q_atm) and the land surface (land_temperature in kelvin,
    saturation); `out` the AtmosphereSurfaceFluxes outputs and interface_temperature."""
    lib = load()
    arrays = {k: state.get(k) for k in F.AL_INPUTS}
    arrays.update({k: out.get(k) for k in F.AL_OUTPUTS})
    arrays["iterations"] = iterations
    f = F.pack(A.ALFields, _grid_of(layout), arrays)
    p = spec.to_c() if hasattr(spec, "to_c") else spec
    o = solver_options(precision)
    st = A.Stats() if stats else None
    ctx = ctx or default_context()
    check(lib.nesf_compute_atmosphere_land_fluxes(ctx.handle, C.byref(p), C.byref(f), C.byref(o),
                                                  C.byref(st) if st is not None else None, _stream_handle(stream)))
    return stats_dict(st) if st is not None else None


def compute_sea_ice_ocean_fluxes(spec, layout, state, out, T3, S3, dz, stream=None, ctx=None):
    """sea_ice_ocean_fluxes.jl:33-77. T3/S3: (nz, ny+2hy, nx+2hx) tensors; T3 is mutated
    by frazil formation; dz: float64 tensor of nz layer thicknesses."""
    lib = load()
    nz = T3.shape[0] if T3.dim() == 3 else 1
    stride_k = T3.shape[-1] * T3.shape[-2]
    p = spec.to_c(nz=nz, stride_k=stride_k) if hasattr(spec, "to_c") else spec
    arrays = {k: state.get(k) for k in ("ice_salinity", "ice_thickness", "consolidation_thickness",
                                        "ice_concentration", "internal_temperature", "ice_mass_flux",
                                        "snow_mass_flux")}
    arrays.update({k: out.get(k) for k in F.IO_OUTPUTS})
    arrays.update(T_oc=T3, S_oc=S3, dz=dz)
    f = F.pack(A.IOFields, _grid_of(layout), arrays)
    check(lib.nesf_compute_sea_ice_ocean_fluxes(ctx.handle if ctx else None, C.byref(p), C.byref(f),
                                                _stream_handle(stream)))


def atmos_grid_struct(atmos):
    La, ca = atmos["layout"], atmos["coords"]
    return A.AtmosGrid(La.nx, La.ny, La.hx, La.hy, La.stride_j, atmos["stride_t"], ca.lon0, ca.dlon, ca.lat0, ca.dlat)


def exchange_coords(c):
    return A.ExchangeCoords(c.lon0, c.dlon, c.lat0, c.dlat)


INTERP_ORDER = ("u", "v", "T", "q", "p", "rain", "snow", "sw", "lw")   # nesf_interp_fields' order
INTERP_SRC = {"u": "u", "v": "v", "T": "T", "q": "q", "p": "p", "rain": "rain", "snow": "snow", "sw": "sw_down",
              "lw": "lw_down"}
INTERP_DST = {"u": "u_out", "v": "v_out", "T": "T_out", "q": "q_out", "p": "p_out", "rain": "rain_out",
              "snow": "snow_out", "sw": "sw_out", "lw": "lw_out"}


def interpolate_atmosphere_state(layout, coords, atmos, atmos_arrays, out, time_weight, frac=None, stream=None):
    """interpolate_atmospheric_state.jl:9-137 + interpolate_radiation_state.jl:4-69.
    `atmos_arrays` maps u v T q p rain snow sw lw to (2, ...) device tensors; `out` maps
    the same names to exchange-grid tensors."""
    lib = load()
    arrays = {}
    for n, t in atmos_arrays.items():
        arrays[INTERP_SRC[n]] = t
    for n, t in out.items():
        arrays[INTERP_DST[n]] = t
    if frac is not None:
        arrays["frac_i"], arrays["frac_j"] = frac
    f = F.pack(A.InterpFields, _grid_of(layout), arrays, coords=exchange_coords(coords),
               atmos=atmos_grid_struct(atmos), time_weight=float(time_weight))
    check(lib.nesf_interpolate_atmosphere_state(C.byref(f), _stream_handle(stream)))


def compute_fractional_indices(layout, coords, atmos, fi, fj, stream=None):
    """prescribed_atmosphere_regridder.jl:41-71 (fi, fj: float64 device tensors)."""
    lib = load()
    g = _grid_of(layout)
    check(lib.nesf_compute_fractional_indices(C.byref(g), C.byref(exchange_coords(coords)),
                                              C.byref(atmos_grid_struct(atmos)), C.c_void_p(fi.data_ptr()),
                                              C.c_void_p(fj.data_ptr()), _stream_handle(stream)))


def _assembly(fn, spec, layout, arrays, stream):
    lib = load()
    f = F.pack(A.AssemblyFields, _grid_of(layout), arrays)
    p = spec.to_c() if hasattr(spec, "to_c") else spec
    check(getattr(lib, fn)(C.byref(p), C.byref(f), _stream_handle(stream)))


def assemble_net_ocean_fluxes(spec, layout, arrays, stream=None):
    """update_net_fluxes!(model, ocean) (assemble_net_ocean_fluxes.jl:30-153)."""
    _assembly("nesf_assemble_net_ocean_fluxes", spec, layout, arrays, stream)


def assemble_net_sea_ice_fluxes(spec, layout, arrays, stream=None):
    """update_net_fluxes!(model, sea_ice) (assemble_net_sea_ice_fluxes.jl:11-81)."""
    _assembly("nesf_assemble_net_sea_ice_fluxes", spec, layout, arrays, stream)


def apply_air_sea_radiative_fluxes(spec, layout, arrays, stream=None):
    """apply_air_sea_radiative_fluxes.jl:18-111."""
    _assembly("nesf_apply_air_sea_radiative_fluxes", spec, layout, arrays, stream)


def apply_air_sea_ice_radiative_fluxes(spec, layout, arrays, stream=None):
    """apply_air_sea_ice_radiative_fluxes.jl:15-90."""
    _assembly("nesf_apply_air_sea_ice_radiative_fluxes", spec, layout, arrays, stream)


def assemble_net_land_fluxes(layout, arrays, stream=None):
    """update_net_fluxes!(model, land::SlabLand) (Lands/slab_land.jl:285-329): `arrays` maps
    nesf_land_flux_fields names to device tensors."""
    lib = load()
    f = F.pack(A.LandFluxFields, _grid_of(layout), arrays)
    check(lib.nesf_assemble_net_land_fluxes(C.byref(f), _stream_handle(stream)))


def apply_air_land_radiative_fluxes(radiation, layout, arrays, stream=None):
    """apply_air_land_radiative_fluxes! (Radiations/apply_air_land_radiative_fluxes.jl:22-95);
    `radiation` is a params.LandRadiation (or an nesf_land_radiation_params)."""
    lib = load()
    f = F.pack(A.LandFluxFields, _grid_of(layout), arrays)
    p = radiation.to_c() if hasattr(radiation, "to_c") else radiation
    check(lib.nesf_apply_air_land_radiative_fluxes(C.byref(p), C.byref(f), _stream_handle(stream)))


def area_integrals(layout, fields, factors=None, inactive=None, area=None, row_area=None, uniform_area=1.0,
                   ctx=None, stream=None):
    """Compensated FP64 area integrals (int dA(a) / int dA(a, b) of the reference's conservation
    checks) of up to 16 device fields; returns a float64 device tensor (n, 2) of (sum, residual)."""
    torch = _torch()
    lib = load()
    n = len(fields)
    factors = factors or [None] * n
    f = A.IntegralFields()
    f.grid = _grid_of(layout)
    f.dtype = A.NESF_F64 if fields[0].dtype == torch.float64 else A.NESF_F32
    f.n = n
    for k in range(n):
        f.field[k] = fields[k].data_ptr()
        f.factor[k] = factors[k].data_ptr() if factors[k] is not None else None
    f.inactive = inactive.data_ptr() if inactive is not None else None
    f.area = area.data_ptr() if area is not None else None
    f.row_area = row_area.data_ptr() if row_area is not None else None
    f.uniform_area = float(uniform_area)
    out = torch.zeros((n, 2), dtype=torch.float64, device=fields[0].device)
    ctx = ctx or default_context()
    check(lib.nesf_area_integrals(ctx.handle, C.byref(f), C.c_void_p(out.data_ptr()), _stream_handle(stream)))
    return out


# ------------------------------------------------------------- coupling step
class CouplingStep:
    """The packed arguments of nesf_coupling_step for one model's fields: the ctypes
    structs are built once and kept alive here, so the device pointers they hold
    stay those of the model's tensors (which must not be reallocated)."""

    def __init__(self, ao_spec, layout, ao_arrays, ai_spec=None, ai_arrays=None, io_spec=None, io_arrays=None,
                 io_levels=(1, 0), interp=None, assembly_spec=None, assembly_arrays=None, radiation=True):
        g = _grid_of(layout)
        self.ao_p = ao_spec.to_c() if hasattr(ao_spec, "to_c") else ao_spec
        self.ao_f = F.pack(A.AOFields, g, ao_arrays)
        self.args = A.CouplingStepArgs()
        self.args.ao_params = C.pointer(self.ao_p)
        self.args.ao = C.pointer(self.ao_f)
        if ai_spec is not None:
            self.ai_p = ai_spec.to_c() if hasattr(ai_spec, "to_c") else ai_spec
            self.ai_f = F.pack(A.AIFields, g, ai_arrays)
            self.args.ai_params = C.pointer(self.ai_p)
            self.args.ai = C.pointer(self.ai_f)
        if io_spec is not None:
            nz, stride_k = io_levels
            self.io_p = io_spec.to_c(nz=nz, stride_k=stride_k) if hasattr(io_spec, "to_c") else io_spec
            self.io_f = F.pack(A.IOFields, g, io_arrays)
            self.args.io_params = C.pointer(self.io_p)
            self.args.io = C.pointer(self.io_f)
        if interp is not None:
            coords, atmos, atmos_arrays, out, frac, tn = interp
            arrays = {INTERP_SRC[n]: t for n, t in atmos_arrays.items()}
            arrays.update({INTERP_DST[n]: t for n, t in out.items()})
            if frac is not None:
                arrays["frac_i"], arrays["frac_j"] = frac
            self.interp_f = F.pack(A.InterpFields, g, arrays, coords=exchange_coords(coords),
                                   atmos=atmos_grid_struct(atmos), time_weight=float(tn))
            self.args.interp = C.pointer(self.interp_f)
        if assembly_spec is not None:
            self.asm_p = assembly_spec.to_c() if hasattr(assembly_spec, "to_c") else assembly_spec
            self.asm_f = F.pack(A.AssemblyFields, g, assembly_arrays)
            self.args.assembly_params = C.pointer(self.asm_p)
            self.args.assembly = C.pointer(self.asm_f)
            self.args.radiation = 1 if radiation else 0

    def set_time_weight(self, tn):
        """Time weight of the interpolation for direct (non-graph) steps."""
        self.interp_f.time_weight = float(tn)


def coupling_step(step, precision="f32_adaptive", ctx=None, stream=None, mlp=None):
    """update_state!'s interface-flux phases in one native call (nesf_coupling_step)."""
    lib = load()
    o = solver_options(precision, mlp=mlp)
    ctx = ctx or default_context()
    check(lib.nesf_coupling_step(ctx.handle, C.byref(step.args), C.byref(o), _stream_handle(stream)))


def get_tuning(ctx=None):
    """The context's launch shapes and schedule (nesf_get_tuning) as a dict."""
    lib = load()
    ctx = ctx or default_context()
    t = A.Tuning()
    check(lib.nesf_get_tuning(ctx.handle, C.byref(t)))
    out = {k: int(getattr(t, k)) for k in A.TUNING_FIELDS}
    out["step_ms"] = float(t.step_ms)
    return out


def set_tuning(ctx=None, **fields):
    """Set fields of the context's tuning (nesf_set_tuning); the others keep their values."""
    lib = load()
    ctx = ctx or default_context()
    cur = get_tuning(ctx)
    unknown = set(fields) - set(A.TUNING_FIELDS)
    if unknown:
        raise ValueError(f"unknown tuning fields {sorted(unknown)}")
    cur.update(fields)
    t = A.Tuning(**{k: int(cur[k]) for k in A.TUNING_FIELDS})
    check(lib.nesf_set_tuning(ctx.handle, C.byref(t)))
    return get_tuning(ctx)


def _tuning_dict(t):
    out = {k: int(getattr(t, k)) for k in A.TUNING_FIELDS}
    out["step_ms"] = float(t.step_ms)
    return out


def autotune(step, precision="f32_adaptive", reps=5, ctx=None, stream=None, mlp=None, cache=None):
    """Coordinate search of the context's tuning on one coupling step (nesf_autotune); returns
    the chosen tuning (a dict with its mean step time, step_ms). The steps run for real.

    `cache`: a tuning-cache file (nesf_autotune_cached). A tuning recorded there for this
    step's key (device, grid, dtype, precision, warm start, phases) is set without running a
    step; otherwise the search runs and its result is recorded. The dict then carries
    "from_cache"."""
    lib = load()
    o = solver_options(precision, mlp=mlp)
    ctx = ctx or default_context()
    t = A.Tuning()
    if cache is None:
        check(lib.nesf_autotune(ctx.handle, C.byref(step.args), C.byref(o), int(reps), C.byref(t),
                                _stream_handle(stream)))
        return _tuning_dict(t)
    hit = C.c_int32(0)
    check(lib.nesf_autotune_cached(ctx.handle, C.byref(step.args), C.byref(o), int(reps), str(cache).encode(),
                                   C.byref(t), C.byref(hit), _stream_handle(stream)))
    out = _tuning_dict(t)
    out["from_cache"] = bool(hit.value)
    return out


def tuning_key(step, precision="f32_adaptive", ctx=None, mlp=None):
    """The tuning-cache key of a coupling step on the context's device (nesf_tuning_key_of)."""
    lib = load()
    o = solver_options(precision, mlp=mlp)
    ctx = ctx or default_context()
    k = A.TuningKey()
    check(lib.nesf_tuning_key_of(ctx.handle, C.byref(step.args), C.byref(o), C.byref(k)))
    return k


def tuning_cache_find(path, key):
    """The tuning a cache file records for `key` (a dict), or None (nesf_tuning_cache_find)."""
    lib = load()
    t = A.Tuning()
    found = C.c_int32(0)
    check(lib.nesf_tuning_cache_find(str(path).encode(), C.byref(key), C.byref(t), C.byref(found)))
    return _tuning_dict(t) if found.value else None


def tuning_cache_store(path, key, tuning):
    """Record `tuning` (a dict of the tuning fields, step_ms optional) for `key`
    (nesf_tuning_cache_store)."""
    lib = load()
    t = A.Tuning(**{k: int(tuning.get(k, 0)) for k in A.TUNING_FIELDS})
    t.step_ms = float(tuning.get("step_ms", 0.0))
    check(lib.nesf_tuning_cache_store(str(path).encode(), C.byref(key), C.byref(t)))


def trace_enable(on=True, ctx=None):
    """Record a kernel-boundary timeline of each coupling step (nesf_trace_enable)."""
    lib = load()
    ctx = ctx or default_context()
    check(lib.nesf_trace_enable(ctx.handle, 1 if on else 0))


def trace_read(ctx=None):
    """The last finished step's marks (nesf_trace_read): a list of (name, stream, t_ms)."""
    lib = load()
    ctx = ctx or default_context()
    buf = (A.TraceEntry * A.TRACE_MAX)()
    n = C.c_int32()
    check(lib.nesf_trace_read(ctx.handle, buf, A.TRACE_MAX, C.byref(n)))
    return [(buf[i].name.decode(), int(buf[i].stream), float(buf[i].t_ms)) for i in range(n.value)]


def timeline(marks):
    """Per-kernel spans (name, stream, start_ms, end_ms) from trace marks: a kernel ends at
    its mark and starts at the previous mark on its stream (the step's start for stream 0;
    None for the first kernel of another stream, which starts when its fork event fires)."""
    last = {}
    spans = []
    for name, stream, t in marks:
        if name == "step":
            last = {0: t}
            continue
        spans.append((name, stream, last.get(stream), t))
        last[stream] = t
    return spans


class Graph:
    """A captured CUDA graph of one coupling step (nesf_graph_capture)."""

    def __init__(self, step, precision="f32_adaptive", ctx=None, mlp=None, calm_replay_wind=None):
        self.lib = load()
        self.step = step                     # keeps the captured pointers' owners alive
        self.mlp = mlp                       # and the network the graph reads
        self.ctx = ctx or default_context()
        o = solver_options(precision, mlp=mlp, calm_replay_wind=calm_replay_wind)
        h = C.c_void_p()
        check(self.lib.nesf_graph_capture(self.ctx.handle, C.byref(step.args), C.byref(o), C.byref(h)))
        self.handle = h

    def set_time_weight(self, tn):
        check(self.lib.nesf_graph_set_time_weight(self.handle, float(tn)))

    def set_forcing(self, arrays, stride_t, tn):
        """nesf_graph_set_forcing: `arrays` maps u v T q p rain snow sw lw to each variable's
        first snapshot (device tensors; absent names keep the captured arrays)."""
        ptrs = (C.c_void_p * 9)(*[(arrays[n].data_ptr() if n in arrays else None) for n in INTERP_ORDER])
        check(self.lib.nesf_graph_set_forcing(self.handle, ptrs, int(stride_t), float(tn)))

    def launch(self, stream=None):
        check(self.lib.nesf_graph_launch(self.handle, _stream_handle(stream)))

    def close(self):
        if self.handle:
            self.lib.nesf_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def to_device(arrays, device="cuda", dtype=None):
    """numpy dict -> torch tensors on the device (uint8/int arrays keep their dtype)."""
    torch = _torch()
    out = {}
    for k, v in arrays.items():
        if v is None:
            out[k] = None
            continue
        t = torch.from_numpy(np.ascontiguousarray(v))
        if dtype is not None and t.is_floating_point():
            t = t.to(dtype)
        out[k] = t.to(device)
    return out
