"""The Julia binding (numericalearth.jl_gb300/julia/NESF.jl) against include/nesf.h.

Julia is not installed here, so the binding cannot run; these tests read it as text
and check what a run would depend on:

* every struct mirror has the C struct's layout: each field at offsetof() of the header
  (compiled here with gcc) and the same size, the Julia layout computed with the C rules
  that Julia's isbits structs follow;
* every `ccall` names an entry point the header declares and the library exports, with
  the prototype's argument count and kinds (pointer / Ref to the matching struct, 32-bit
  integer, double) and return type;
* every phase of update_state! that the interface-flux step covers
  (time_step_earth_system_model.jl:50-80) has a method taking the coupled model alone, or
  with its component, specialised on the model type that carries the wrapper.
"""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from nesf import _lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "nesf.h")
SHIM = os.path.join(REPO, "numericalearth.jl_gb300", "julia", "NESF.jl")

JULIA_TO_C = {
    "Grid": "nesf_grid", "ThermodynamicsParameters": "nesf_thermodynamics_parameters",
    "StabilityFunction": "nesf_stability_function", "RoughnessLength": "nesf_roughness_length",
    "SimilarityTheoryFluxesC": "nesf_similarity_theory_fluxes", "CoefficientFluxes": "nesf_coefficient_fluxes",
    "InterfaceParams": "nesf_interface_params", "SolverOptions": "nesf_solver_options",
    "AOFields": "nesf_ao_fields", "ALFields": "nesf_al_fields", "AIFields": "nesf_ai_fields",
    "IOParams": "nesf_io_params", "IOFields": "nesf_io_fields", "AtmosGrid": "nesf_atmos_grid",
    "ExchangeCoords": "nesf_exchange_coords", "InterpFields": "nesf_interp_fields",
    "AssemblyParams": "nesf_assembly_params", "AssemblyFields": "nesf_assembly_fields",
}
SCALARS = {"Int32": 4, "UInt32": 4, "Cint": 4, "Int64": 8, "UInt64": 8, "Float64": 8, "Float32": 4, "UInt8": 1}


def shim_text():
    return open(SHIM).read()


def julia_structs():
    """name -> [(field, type)] of the isbits struct mirrors."""
    out = {}
    for name, body in re.findall(r"^struct (\w+)\n(.*?)^end", shim_text(), re.S | re.M):
        if name not in JULIA_TO_C:
            continue
        fields = []
        for part in re.split(r"[;\n]", body):
            part = part.split("#")[0].strip()
            if part:
                f, t = part.split("::")
                fields.append((f.strip(), t.strip()))
        out[name] = fields
    return out


def layout(jtype, structs, cache):
    """(size, alignment) of a Julia field type under the C layout rules."""
    if jtype in SCALARS:
        return SCALARS[jtype], SCALARS[jtype]
    if jtype.startswith("Ptr{"):
        return 8, 8
    m = re.fullmatch(r"NTuple\{(\d+), (\w+)\}", jtype)
    if m:
        size, align = layout(m.group(2), structs, cache)
        return int(m.group(1)) * size, align
    return struct_layout(jtype, structs, cache)[:2]


def struct_layout(name, structs, cache):
    """(size, alignment, {field: offset}) of a mirror."""
    if name in cache:
        return cache[name]
    off, align, offsets = 0, 1, {}
    for f, t in structs[name]:
        size, a = layout(t, structs, cache)
        off = (off + a - 1) // a * a
        offsets[f] = off
        off += size
        align = max(align, a)
    size = (off + align - 1) // align * align
    cache[name] = (size, align, offsets)
    return cache[name]


def compile_and_run(tmp_path, lines):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "probe.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "nesf.h"\nint main(void) {\n' +
                   "".join(lines) + "    return 0;\n}\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-I", os.path.dirname(HEADER), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict(line.split() for line in out.splitlines())


def test_every_struct_mirror_has_the_header_layout(tmp_path):
    structs = julia_structs()
    assert set(structs) == set(JULIA_TO_C), set(JULIA_TO_C) - set(structs)
    lines = []
    for jname, cname in JULIA_TO_C.items():
        lines.append(f'    printf("{jname}.__size__ %zu\\n", sizeof({cname}));\n')
        for f, _ in structs[jname]:
            lines.append(f'    printf("{jname}.{f} %zu\\n", offsetof({cname}, {f}));\n')
    c = compile_and_run(tmp_path, lines)
    cache = {}
    for jname in JULIA_TO_C:
        size, _, offsets = struct_layout(jname, structs, cache)
        assert int(c[f"{jname}.__size__"]) == size, jname
        for f, off in offsets.items():
            assert int(c[f"{jname}.{f}"]) == off, (jname, f)


def header_prototypes():
    """name -> (return type, [argument types]) of the header's functions."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for ret, name, args in re.findall(r"^\s*([\w\s\*]+?)\s*\b(nesf_\w+)\s*\(([^;{]*?)\)\s*;", text, re.M | re.S):
        arglist = [] if args.strip() in ("", "void") else [" ".join(a.split()) for a in args.split(",")]
        types = []
        for a in arglist:
            a = re.sub(r"\b\w+$", "", a).strip() if not a.endswith("*") else a
            types.append(a)
        protos[name] = (" ".join(ret.split()), types)
    return protos


def c_kind(ctype):
    """The kind of a C argument type: ('ptr', struct name or scalar), ('int32',), ('double',) ..."""
    t = ctype.replace("const ", "").strip()
    if t.endswith("*"):
        base = t[:-1].strip().rstrip("*").strip()
        return ("ptr", base)
    return {"int32_t": ("int32",), "int": ("int32",), "double": ("double",), "int64_t": ("int64",),
            "uint64_t": ("int64",)}.get(t, ("other", t))


def julia_kind(jtype):
    jtype = jtype.strip()
    m = re.fullmatch(r"(?:Ref|Ptr)\{(\w+)\}", jtype)
    if m:
        inner = m.group(1)
        c = JULIA_TO_C.get(inner) or {"Cvoid": "void", "UInt8": "uint8_t", "Int32": "int32_t", "Float64": "double"
                                      }.get(inner, inner)
        return ("ptr", c)
    return {"Int32": ("int32",), "Cint": ("int32",), "Float64": ("double",), "Int64": ("int64",),
            "UInt64": ("int64",)}.get(jtype, ("other", jtype))


def split_top(s):
    """Split a comma list at depth 0 of (), {}."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def shim_ccalls():
    """[(function name, return type, [argument types])] of the shim's ccalls; the assembly
    entries run through run_assembly!(model, :name) with its one signature."""
    text = shim_text()
    calls = []
    for m in re.finditer(r"ccall\(\((:?\w+), libnesf\),\s*(\w+),\s*\(", text):
        i = m.end()
        depth, j = 1, i
        while depth:
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        types = split_top(text[i:j - 1])
        name = m.group(1)
        calls.append((name.lstrip(":"), m.group(2), types))
    generic = [c for c in calls if c[0] == "entry"]
    assert len(generic) == 1
    for name in re.findall(r"run_assembly!\(model, :(\w+)\)", text):
        calls.append((name, generic[0][1], generic[0][2]))
    return [c for c in calls if c[0] != "entry"]


def test_every_ccall_matches_its_prototype():
    protos = header_prototypes()
    lib = C.CDLL(_lib.LIB_PATH if os.path.exists(_lib.LIB_PATH) else _lib.load()._name)
    calls = shim_ccalls()
    names = {c[0] for c in calls}
    assert {"nesf_compute_atmosphere_ocean_fluxes", "nesf_compute_atmosphere_sea_ice_fluxes",
            "nesf_compute_sea_ice_ocean_fluxes", "nesf_interpolate_atmosphere_state", "nesf_time_indices",
            "nesf_assemble_net_ocean_fluxes", "nesf_assemble_net_sea_ice_fluxes",
            "nesf_apply_air_sea_radiative_fluxes", "nesf_apply_air_sea_ice_radiative_fluxes",
            "nesf_compute_atmosphere_land_fluxes"} <= names
    for name, ret, jargs in calls:
        assert name in protos, name
        assert hasattr(lib, name), name
        cret, cargs = protos[name]
        assert len(jargs) == len(cargs), (name, jargs, cargs)
        assert {"Cint": "int", "Cvoid": "void", "Cstring": "const char*"}[ret] == cret.replace(" *", "*"), (name, ret)
        for ja, ca in zip(jargs, cargs):
            jk, ck = julia_kind(ja), c_kind(ca)
            if jk[0] == "ptr" and ck[0] == "ptr" and (jk[1] == "void" or ck[1] == "void"):
                continue   # an opaque pointer on either side (context, stream, device data)
            assert jk == ck, (name, ja, ca)


def test_update_state_phases_have_methods_for_the_wrapped_model():
    """The methods update_state! reaches with the coupled model alone (or with its component)."""
    text = shim_text()
    assert re.search(r"const GB300Model = EarthSystemModel\{<:Any, <:Any, <:Any, <:Any, <:Any, <:GB300Interfaces\}",
                     text)
    assert "const GB300Interfaces = IC.ComponentInterfaces{<:GB300AOInterface}" in text
    for sig in (r"function IC\.compute_atmosphere_ocean_fluxes!\(model::GB300Model\)",
                r"function IC\.compute_atmosphere_sea_ice_fluxes!\(model::GB300Model\)",
                r"function IC\.compute_sea_ice_ocean_fluxes!\(model::GB300Model\)",
                r"function ESM\.interpolate_state!\(exchanger, grid::LatitudeLongitudeGrid, "
                r"atmosphere::PrescribedAtmosphere,\s*model::GB300Model\)",
                r"ESM\.update_net_fluxes!\(model::GB300Model, ocean::",
                r"ESM\.update_net_fluxes!\(model::GB300Model, sea_ice::Simulation\{<:SeaIceModel\}\)",
                r"function ESM\.apply_air_sea_radiative_fluxes!\(model::GB300Model\)",
                r"function ESM\.apply_air_sea_ice_radiative_fluxes!\(model::GB300Model\)"):
        assert re.search(sig, text), sig
    # the packers read the wrapped formulation's own fields, not library defaults alone
    for field in ("von_karman_constant", "turbulent_prandtl_number", "solver_stop_criteria", "roughness_lengths",
                  "stability_functions", "boundary_layer_height", "surface_layer_height",
                  "specific_humidity_formulation", "temperature_formulation"):
        assert field in text, field
