"""Packing of arrays into the field-bundle structs of include/nesf.h.

Arrays may be torch CUDA tensors (the library path) or numpy arrays (the
oracle path on the host). Every 2-D array of one call must share the grid
layout `(ny + 2hy, nx + 2hx)` with i fastest.
"""
import ctypes as C

import numpy as np

from . import _abi as A


def pointer(a):
    """Raw data pointer of a torch tensor or numpy array (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)!r}")


def dtype_code(a):
    name = str(a.dtype)
    if name.endswith("float64"):
        return A.NESF_F64
    if name.endswith("float32"):
        return A.NESF_F32
    raise TypeError(f"unsupported dtype {a.dtype}")


def make_grid(layout):
    return A.Grid(layout.nx, layout.ny, layout.hx, layout.hy, layout.stride_j)


def pack(struct_cls, grid, arrays, dtype=None, **extra):
    """Fill a bundle: `grid` is an nesf_grid, `arrays` maps field names to arrays."""
    s = struct_cls()
    names = {n for n, _ in struct_cls._fields_}
    if "grid" in names:
        s.grid = grid
    ref_dtype = None
    for k, v in arrays.items():
        if k not in names:
            raise KeyError(f"{struct_cls.__name__} has no field {k!r}")
        setattr(s, k, pointer(v))
        if v is not None and k not in ("inactive", "iterations", "dz", "frac_i", "frac_j"):
            code = dtype_code(v)
            if ref_dtype is None:
                ref_dtype = code
            elif code != ref_dtype:
                raise TypeError(f"{k}: all float arrays of one call must share a dtype")
    if "dtype" in names:
        s.dtype = ref_dtype if dtype is None else dtype
    for k, v in extra.items():
        setattr(s, k, v)
    return s


AO_INPUTS = ("u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "u_oc", "v_oc", "T_oc", "S_oc", "inactive",
             "sw_down", "lw_down", "kappa")
AO_OUTPUTS = ("latent_heat", "sensible_heat", "water_vapor", "x_momentum", "y_momentum",
              "friction_velocity", "temperature_scale", "water_vapor_scale", "interface_temperature")
AI_INPUTS = ("u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "T_oc", "S_oc", "ice_thickness", "snow_thickness",
             "consolidation_thickness", "ice_concentration", "inactive", "sw_down", "lw_down")
AI_OUTPUTS = ("latent_heat", "sensible_heat", "water_vapor", "x_momentum", "y_momentum")
IO_OUTPUTS = ("interface_heat", "frazil_heat", "salt", "freshwater", "interface_T", "interface_S")
AL_INPUTS = ("u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "land_temperature", "saturation")
AL_OUTPUTS = AO_OUTPUTS
