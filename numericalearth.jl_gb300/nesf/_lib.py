"""Loader of libnesf.so with the ctypes signatures of include/nesf.h.

The library is required: there is no CPU fallback. `load()` raises if the
shared library is missing or does not export the full ABI.
"""
import ctypes as C
import os
import threading

from . import _abi as A

_LIB = None
_LOCK = threading.Lock()

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libnesf.so")

P = C.POINTER
vp = C.c_void_p

# name -> (restype, argtypes); the exact entry points declared in include/nesf.h
SIGNATURES = {
    "nesf_abi_version": (C.c_int32, []),
    "nesf_version": (C.c_char_p, []),
    "nesf_last_error": (C.c_char_p, []),
    "nesf_struct_sizes": (C.c_int32, [P(C.c_int64), C.c_int32]),
    "nesf_default_thermodynamics": (None, [P(A.ThermodynamicsParameters)]),
    "nesf_default_ao_params": (None, [P(A.InterfaceParams)]),
    "nesf_default_ai_params": (None, [P(A.InterfaceParams)]),
    "nesf_default_al_params": (None, [P(A.InterfaceParams)]),
    "nesf_default_coefficient_fluxes": (None, [P(A.CoefficientFluxes), C.c_int32]),
    "nesf_default_io_params": (None, [P(A.IOParams)]),
    "nesf_time_indices": (C.c_int, [P(C.c_double), C.c_int32, C.c_int32, C.c_double, C.c_double, P(C.c_int32),
                                          P(C.c_int32), P(C.c_double)]),
    "nesf_init": (C.c_int, [C.c_int32]),
    "nesf_default_assembly_params": (None, [P(A.AssemblyParams)]),
    "nesf_default_solver_options": (None, [P(A.SolverOptions)]),
    "nesf_context_create": (C.c_int, [C.c_int32, P(vp)]),
    "nesf_context_destroy": (C.c_int, [vp]),
    "nesf_compute_atmosphere_ocean_fluxes": (
        C.c_int, [vp, P(A.InterfaceParams), P(A.AOFields), P(A.SolverOptions), P(A.Stats), vp]),
    "nesf_compute_atmosphere_ocean_fluxes_ensemble": (
        C.c_int, [vp, P(A.InterfaceParams), C.c_int32, C.c_int64, P(A.AOFields), P(A.SolverOptions),
                  P(A.Stats), vp]),
    "nesf_compute_atmosphere_ocean_fluxes_noalloc": (
        C.c_int, [P(A.InterfaceParams), P(A.AOFields), P(A.SolverOptions), vp]),
    "nesf_noalloc_prepare": (C.c_int, [C.c_int32]),
    "nesf_compute_atmosphere_sea_ice_fluxes": (
        C.c_int, [vp, P(A.InterfaceParams), P(A.AIFields), P(A.SolverOptions), P(A.Stats), vp]),
    "nesf_compute_atmosphere_land_fluxes": (
        C.c_int, [vp, P(A.InterfaceParams), P(A.ALFields), P(A.SolverOptions), P(A.Stats), vp]),
    "nesf_compute_sea_ice_ocean_fluxes": (C.c_int, [vp, P(A.IOParams), P(A.IOFields), vp]),
    "nesf_compute_fractional_indices": (
        C.c_int, [P(A.Grid), P(A.ExchangeCoords), P(A.AtmosGrid), vp, vp, vp]),
    "nesf_interpolate_atmosphere_state": (C.c_int, [P(A.InterpFields), vp]),
    "nesf_assemble_net_ocean_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields), vp]),
    "nesf_assemble_net_sea_ice_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields), vp]),
    "nesf_apply_air_sea_radiative_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields), vp]),
    "nesf_apply_air_sea_ice_radiative_fluxes": (C.c_int, [P(A.AssemblyParams), P(A.AssemblyFields), vp]),
    "nesf_assemble_net_land_fluxes": (C.c_int, [P(A.LandFluxFields), vp]),
    "nesf_apply_air_land_radiative_fluxes": (C.c_int, [P(A.LandRadiationParams), P(A.LandFluxFields), vp]),
    "nesf_area_integrals": (C.c_int, [vp, P(A.IntegralFields), vp, vp]),
    "nesf_mlp_selftest": (C.c_int, [vp, vp, vp, C.c_int32, vp]),
    "nesf_double_float_check": (C.c_int, [vp, vp, vp, C.c_int64, C.c_int32, vp]),
    "nesf_mlp_bytes": (C.c_int64, []),
    "nesf_mlp_init": (C.c_int, [vp, C.c_uint64, vp]),
    "nesf_mlp_fit_normalization": (C.c_int, [vp, vp, vp, C.c_int64, vp]),
    "nesf_mlp_gradient": (C.c_int, [vp, vp, vp, C.c_int64, vp]),
    "nesf_mlp_train": (C.c_int, [vp, vp, vp, C.c_int64, P(A.MlpTrainOptions), P(C.c_float), vp]),
    "nesf_mlp_infer": (C.c_int, [vp, vp, C.c_int64, vp, vp]),
    "nesf_mlp_ao_samples": (C.c_int, [P(A.InterfaceParams), P(A.AOFields), vp, vp, vp]),
    "nesf_coupling_step": (C.c_int, [vp, P(A.CouplingStepArgs), P(A.SolverOptions), vp]),
    "nesf_graph_capture": (C.c_int, [vp, P(A.CouplingStepArgs), P(A.SolverOptions), P(vp)]),
    "nesf_graph_set_time_weight": (C.c_int, [vp, C.c_double]),
    "nesf_graph_set_forcing": (C.c_int, [vp, P(vp), C.c_int64, C.c_double]),
    "nesf_graph_launch": (C.c_int, [vp, vp]),
    "nesf_graph_destroy": (C.c_int, [vp]),
    "nesf_set_tuning": (C.c_int, [vp, P(A.Tuning)]),
    "nesf_get_tuning": (C.c_int, [vp, P(A.Tuning)]),
    "nesf_autotune": (C.c_int, [vp, P(A.CouplingStepArgs), P(A.SolverOptions), C.c_int32, P(A.Tuning), vp]),
    "nesf_tuning_key_of": (C.c_int, [vp, P(A.CouplingStepArgs), P(A.SolverOptions), P(A.TuningKey)]),
    "nesf_tuning_cache_find": (C.c_int, [C.c_char_p, P(A.TuningKey), P(A.Tuning), P(C.c_int32)]),
    "nesf_tuning_cache_store": (C.c_int, [C.c_char_p, P(A.TuningKey), P(A.Tuning)]),
    "nesf_autotune_cached": (C.c_int, [vp, P(A.CouplingStepArgs), P(A.SolverOptions), C.c_int32, C.c_char_p,
                                       P(A.Tuning), P(C.c_int32), vp]),
    "nesf_trace_enable": (C.c_int, [vp, C.c_int32]),
    "nesf_trace_read": (C.c_int, [vp, P(A.TraceEntry), C.c_int32, P(C.c_int32)]),
}


class NesfError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"nesf error {code}: {message}")
        self.code = code


def load(path=None):
    """Load libnesf.so (building it first if it is missing and nvcc is present)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = path or LIB_PATH
        if not os.path.exists(path):
            from . import build
            build.build()
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)   # AttributeError = missing export: fail loudly
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def check(code):
    if code != A.NESF_OK:
        msg = load().nesf_last_error().decode(errors="replace")
        raise NesfError(code, msg)
    return code
