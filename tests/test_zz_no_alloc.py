"""The allocation-free atmosphere-ocean entry point against the regular one.

nesf_compute_atmosphere_ocean_fluxes_noalloc is for callers that cannot allocate
device memory when the flux step runs (a host model whose pooling allocator holds
the whole device, or a caller that must not enter the driver's allocator). It
keeps its scratch in a fixed array inside the library, which nesf_noalloc_prepare
sets up once per device. The tests:

* call it through the C ABI twice in a row -- the second call finds the previous
  call's work list and replay queue in the shared scratch -- and check both calls
  against nesf_compute_atmosphere_ocean_fluxes on the same inputs, with the
  tolerance of the other GPU tests (relative error |a - b| / max(|b|, 1e-6 max|b|)
  <= 1e-12) for the FP64 and FP32 solvers; under the adaptive FP32 solver the
  regular entry point's pass 1 reads its cancelling differences from the classify
  pass's double-float records, a scratch this entry point does not hold (it forms
  them in FP64 in the kernel), so the two FP32 trajectories differ and agree within
  twice the solver's tolerance against FP64 (2e-5), while the two calls agree bit
  for bit;
* check that the device's free memory (cudaMemGetInfo) is the same before and
  after those calls: they allocate nothing;
* run a grid whose halo ring is exactly the scratch capacity (2^21 cells) and
  check that one row more is refused before any launch;
* check that a warm start, whose buffers would be allocated, is refused.

This file is collected last so that a failing run stopped at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_err, to_numpy
from nesf import _abi as A
from nesf import _lib, api
from nesf import fields as F
from nesf import params as P
from nesf import synthetic as syn

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 21


def _noalloc(lib, spec, layout, dev, out, precision, mlp=None):
    import torch
    arrays = {k: dev.get(k) for k in F.AO_INPUTS}
    arrays.update({k: out[k] for k in F.AO_OUTPUTS})
    f = F.pack(A.AOFields, F.make_grid(layout), arrays)
    p = spec.to_c()
    o = api.solver_options(precision)
    if mlp is not None:
        o.warm_start = 1
        o.mlp = mlp.data_ptr()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib.nesf_compute_atmosphere_ocean_fluxes_noalloc(C.byref(p), C.byref(f), C.byref(o), stream)


def _prepare(lib):
    import torch
    code = lib.nesf_noalloc_prepare(torch.cuda.current_device())
    assert code == A.NESF_OK, lib.nesf_last_error()


@pytest.mark.parametrize("precision,dtype", [("f64", np.float64), ("f32", np.float32), ("f32_adaptive", np.float32)])
def test_noalloc_matches_regular_entry_point_twice(precision, dtype):
    import torch
    lib = _lib.load()
    _prepare(lib)
    st = syn.coupled(seed=31, nx=360, ny=160, lat_s=-75, lat_n=75, land=0.3, interpolate=False, dtype=dtype)
    spec = P.atmosphere_ocean_interface_spec()
    dev = api.to_device({k: st.fields[k] for k in F.AO_INPUTS if k in st.fields})
    fdt = dev["u_atm"].dtype
    ref = {k: torch.zeros(st.layout.shape, dtype=fdt, device="cuda") for k in F.AO_OUTPUTS}
    api.compute_atmosphere_ocean_fluxes(spec, st.layout, dev, ref, precision=precision)
    torch.cuda.synchronize()
    R = st.layout.ring
    expect = {k: R(to_numpy(v)).astype(np.float64) for k, v in ref.items()}
    outs = [{k: torch.full(st.layout.shape, float("nan"), dtype=fdt, device="cuda") for k in F.AO_OUTPUTS}
            for _ in range(2)]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for call in range(2):
        code = _noalloc(lib, spec, st.layout, dev, outs[call], precision)
        assert code == A.NESF_OK, lib.nesf_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free calls changed the free device memory"
    tol = 2e-5 if precision == "f32_adaptive" else 1e-12
    for call in range(2):
        for k in F.AO_OUTPUTS:
            got = R(to_numpy(outs[call][k])).astype(np.float64)
            e = rel_err(got, expect[k], floor_frac=1e-6)
            assert e.max() <= tol, (precision, call, k, float(e.max()))
    for k in F.AO_OUTPUTS:   # (cells the solve does not write keep their NaN)
        assert np.array_equal(to_numpy(outs[0][k]), to_numpy(outs[1][k]), equal_nan=True), (precision, k)


def test_noalloc_at_capacity_and_beyond():
    """A grid of exactly 2^21 halo-ring cells (2046 x 1022) is solved and matches the regular
    entry point (adaptive FP32 solver: within 2e-5, as above); one row more is refused with
    NESF_ERR_CAPACITY before any launch."""
    import torch
    lib = _lib.load()
    _prepare(lib)
    nx, ny = 2046, 1022
    assert (nx + 2) * (ny + 2) == MAX_CELLS
    st = syn.coupled(seed=33, nx=nx, ny=ny, lat_s=-75, lat_n=75, land=0.3, interpolate=False, dtype=np.float32)
    spec = P.atmosphere_ocean_interface_spec()
    dev = api.to_device({k: st.fields[k] for k in F.AO_INPUTS if k in st.fields})
    ref = {k: torch.zeros(st.layout.shape, dtype=torch.float32, device="cuda") for k in F.AO_OUTPUTS}
    api.compute_atmosphere_ocean_fluxes(spec, st.layout, dev, ref, precision="f32_adaptive")
    out = {k: torch.full(st.layout.shape, float("nan"), dtype=torch.float32, device="cuda") for k in F.AO_OUTPUTS}
    code = _noalloc(lib, spec, st.layout, dev, out, "f32_adaptive")
    assert code == A.NESF_OK, lib.nesf_last_error()
    torch.cuda.synchronize()
    R = st.layout.ring
    for k in F.AO_OUTPUTS:
        e = rel_err(R(to_numpy(out[k])).astype(np.float64), R(to_numpy(ref[k])).astype(np.float64), floor_frac=1e-6)
        assert e.max() <= 2e-5, (k, float(e.max()))
    over = syn.Layout(nx, ny + 1, st.layout.hx, st.layout.hy)
    assert (nx + 2) * (ny + 3) > MAX_CELLS
    code = _noalloc(lib, spec, over, dev, out, "f32_adaptive")
    assert code == A.NESF_ERR_CAPACITY
    assert b"exceed" in lib.nesf_last_error()


def test_noalloc_refuses_grids_beyond_its_scratch():
    import torch
    lib = _lib.load()
    _prepare(lib)
    spec = P.atmosphere_ocean_interface_spec()
    nx, ny = 2048, 1024                     # (nx + 2) * (ny + 2) > 2**21
    assert (nx + 2) * (ny + 2) > MAX_CELLS
    layout = syn.Layout(nx, ny, 2, 2)
    small = torch.zeros(16, dtype=torch.float64, device="cuda")   # never read: refused before any launch
    arrays = {k: small for k in ("u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "u_oc", "v_oc", "T_oc", "S_oc")}
    arrays.update({k: small for k in F.AO_OUTPUTS})
    code = _noalloc(lib, spec, layout, arrays, arrays, "f64")
    assert code == A.NESF_ERR_CAPACITY
    assert b"exceed" in lib.nesf_last_error()


def test_noalloc_refuses_a_warm_start():
    import torch
    lib = _lib.load()
    _prepare(lib)
    st = syn.ao_1deg(seed=35, nx=32, ny=16)
    spec = P.atmosphere_ocean_interface_spec()
    dev = api.to_device({k: st.fields[k] for k in F.AO_INPUTS if k in st.fields})
    out = {k: torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda") for k in F.AO_OUTPUTS}
    blob = torch.zeros(lib.nesf_mlp_bytes(), dtype=torch.uint8, device="cuda")   # never read: refused first
    code = _noalloc(lib, spec, st.layout, dev, out, "f32_adaptive", mlp=blob)
    assert code == A.NESF_ERR_ARG
    assert b"warm start" in lib.nesf_last_error()
