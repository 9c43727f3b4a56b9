"""libnesf.so loads without a GPU, exports every entry point of include/nesf.h,
and its struct layouts agree with the Python bindings."""
import ctypes as C
import os
import re

import pytest

from nesf import _abi as A
from nesf import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "nesf.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nesf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_entry_point():
    lib = C.CDLL(_lib.LIB_PATH if os.path.exists(_lib.LIB_PATH) else _lib.load()._name)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_struct_sizes_match_bindings():
    lib = _lib.load()
    n = len(A.STRUCTS_IN_SIZE_ORDER)
    sizes = (C.c_int64 * n)()
    m = lib.nesf_struct_sizes(sizes, n)
    assert m == n
    for k, cls in enumerate(A.STRUCTS_IN_SIZE_ORDER):
        assert sizes[k] == C.sizeof(cls), cls.__name__


def test_defaults_match_reference_constructors():
    """The library's defaults equal the Python mirror of the reference constructors."""
    from nesf import params as P
    lib = _lib.load()
    ao = A.InterfaceParams()
    lib.nesf_default_ao_params(C.byref(ao))
    mine = P.atmosphere_ocean_interface_spec().to_c()
    assert bytes(ao) == bytes(mine)
    ai = A.InterfaceParams()
    lib.nesf_default_ai_params(C.byref(ai))
    mine = P.atmosphere_sea_ice_interface_spec().to_c()
    assert bytes(ai) == bytes(mine)
    io = A.IOParams()
    lib.nesf_default_io_params(C.byref(io))
    assert bytes(io) == bytes(P.SeaIceOceanSpec().to_c())
    ap = A.AssemblyParams()
    lib.nesf_default_assembly_params(C.byref(ap))
    assert bytes(ap) == bytes(P.AssemblySpec().to_c())


def test_argument_errors_without_gpu():
    """Bad arguments are rejected on the host before any device work."""
    lib = _lib.load()
    p = A.InterfaceParams()
    lib.nesf_default_ao_params(C.byref(p))
    f = A.AOFields()
    f.grid = A.Grid(10, 10, 1, 1, 12)     # halo 1 is too small for the face averages
    f.dtype = A.NESF_F64
    code = lib.nesf_compute_atmosphere_ocean_fluxes(None, C.byref(p), C.byref(f), None, None, None)
    assert code == A.NESF_ERR_ARG
    assert b"halo" in lib.nesf_last_error()
    f.grid = A.Grid(10, 10, 2, 2, 14)
    code = lib.nesf_compute_atmosphere_ocean_fluxes(None, C.byref(p), C.byref(f), None, None, None)
    assert code == A.NESF_ERR_ARG and b"u_atm" in lib.nesf_last_error()
    p.fluxes.maxiter = -1
    code = lib.nesf_compute_atmosphere_ocean_fluxes(None, C.byref(p), C.byref(f), None, None, None)
    assert code == A.NESF_ERR_ARG and b"maxiter" in lib.nesf_last_error()
    assert lib.nesf_abi_version() == 1
    with pytest.raises(_lib.NesfError):
        _lib.check(A.NESF_ERR_ARG)


def test_network_blob_layout_matches_binding():
    lib = _lib.load()
    assert lib.nesf_mlp_bytes() == C.sizeof(A.MlpBlob)


@pytest.mark.parametrize("field,value", [("solve_block", 48), ("solve_block", 160), ("deferred_per_sm", 17),
                                         ("infer_per_sm", -1), ("two_lanes", 2), ("io_overlap", -1),
                                         ("pass1_fetch", 5), ("pass1_fetch", -1), ("refill_lanes", 33),
                                         ("refill_lanes", -2)])
def test_tuning_out_of_range_is_an_argument_error(field, value):
    """nesf_set_tuning checks its fields before it touches a device."""
    lib = _lib.load()
    t = A.Tuning(**{field: value})
    assert lib.nesf_set_tuning(None, C.byref(t)) == A.NESF_ERR_ARG
    assert field in lib.nesf_last_error().decode()


def test_work_table_matches_header():
    """The roofline's work-per-unit table (NESF_WORK_*) as the Python side reads it."""
    text = open(HEADER).read()
    found = dict(re.findall(r"#define NESF_WORK_([A-Z0-9_]+)\s+(\d+)", text))
    assert {k: int(v) for k, v in found.items()} == A.WORK


# include/nesf.h's structs in the order of nesf_struct_sizes() and of A.STRUCTS_IN_SIZE_ORDER
C_STRUCT_NAMES = (
    "nesf_grid", "nesf_thermodynamics_parameters", "nesf_stability_function", "nesf_roughness_length",
    "nesf_similarity_theory_fluxes", "nesf_interface_params", "nesf_solver_options", "nesf_stats",
    "nesf_ao_fields", "nesf_ai_fields", "nesf_io_params", "nesf_io_fields", "nesf_atmos_grid",
    "nesf_exchange_coords", "nesf_interp_fields", "nesf_assembly_params", "nesf_assembly_fields",
    "nesf_coupling_step_args", "nesf_integral_fields", "nesf_tuning", "nesf_trace_entry",
    "nesf_coefficient_fluxes", "nesf_al_fields", "nesf_land_radiation_params", "nesf_land_flux_fields",
    "nesf_tuning_key")


@pytest.mark.parametrize("k", range(len(C_STRUCT_NAMES)))
def test_struct_field_offsets_match_header(tmp_path, k):
    """Every field of each ctypes mirror sits at offsetof() of include/nesf.h (compiled here)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    assert len(C_STRUCT_NAMES) == len(A.STRUCTS_IN_SIZE_ORDER)
    c_name, mirror = C_STRUCT_NAMES[k], A.STRUCTS_IN_SIZE_ORDER[k]
    names = [f[0] for f in mirror._fields_]
    src = tmp_path / "off.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "nesf.h"\nint main(void) {\n' +
                   "".join(f'    printf("{k} %zu\\n", offsetof({c_name}, {k}));\n' for k in names) +
                   "    return 0;\n}\n")
    exe = tmp_path / "off"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), "-o", str(exe), str(src)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                      text=True).stdout.splitlines())
    for k in names:
        assert int(out[k]) == getattr(mirror, k).offset, (c_name, k)


def test_mlp_entry_points_refuse_misaligned_features():
    """The network's passes read each sample's 8 features as two 16-byte vectors: a feature
    pointer off a 16-byte boundary is refused before any device work (checked here with
    placeholder addresses that are never dereferenced)."""
    import ctypes as C
    lib = _lib.load()
    blob, out, targets = C.c_void_p(0x10000), C.c_void_p(0x20000), C.c_void_p(0x30000)
    misaligned = C.c_void_p(0x40004)
    assert lib.nesf_mlp_infer(blob, misaligned, 128, out, None) == A.NESF_ERR_ARG
    assert b"16-byte" in lib.nesf_last_error()
    assert lib.nesf_mlp_gradient(blob, misaligned, targets, 128, None) == A.NESF_ERR_ARG
    o = A.MlpTrainOptions(1, 128, 1e-3, 0.9, 0.999, 1e-8)
    assert lib.nesf_mlp_train(blob, misaligned, targets, 128, C.byref(o), None, None) == A.NESF_ERR_ARG
