"""Sea-ice interfaces, interpolation and net-flux assembly on the GPU against the oracle.

Relative errors are |gpu - ref| / max(|ref|, 1e-6 max|ref|) (see test_gpu_ao.py):
1e-12 for FP64 kernels, 1e-5 for the FP32 + FP64-polish solve."""
import numpy as np
import pytest

from helpers import rel_err, to_numpy, widen
from nesf import api
from nesf import fields as F
from nesf import params as P
from nesf import synthetic as syn

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def coupled64():
    return syn.coupled(seed=21, nx=120, ny=64, lat_s=-80, lat_n=80, land=0.2, interpolate=False, dtype=np.float64)


def run_ai(spec, st, precision="f64"):
    import torch
    dev = api.to_device({k: st.fields.get(k) for k in F.AI_INPUTS if k in st.fields})
    fdt = dev["u_atm"].dtype
    out = {k: torch.zeros(st.layout.shape, dtype=fdt, device="cuda") for k in F.AI_OUTPUTS}
    out["interface_temperature"] = api.to_device({"t": st.fields["ice_temperature"]})["t"].clone()
    it = torch.zeros(st.layout.shape, dtype=torch.int32, device="cuda")
    api.compute_atmosphere_sea_ice_fluxes(spec, st.layout, dev, out, precision=precision, iterations=it)
    torch.cuda.synchronize()
    res = {k: to_numpy(v) for k, v in out.items()}
    res["iterations"] = to_numpy(it)
    return res


def test_atmosphere_sea_ice_plain_matches_oracle(oracle, coupled64):
    st = coupled64
    spec = P.atmosphere_sea_ice_interface_spec()
    ref = oracle.ai_fluxes(spec.to_c(), st.layout, st.fields, st.fields["ice_temperature"])
    gpu = run_ai(spec, st, "f64")
    R = st.layout.ring
    ice = R(st.fields["ice_concentration"]) > 0
    assert ice.sum() > 100
    for k in F.AI_OUTPUTS:
        e = rel_err(R(gpu[k]), R(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-12, (k, e.max())
    # the interface temperature is compared in kelvin: stored in Celsius, a 1-ulp
    # difference of T [K] is a large relative error of T [C] near the melting point
    e = rel_err(R(gpu["interface_temperature"]) + 273.15, R(ref["interface_temperature"]) + 273.15)
    assert e.max() <= 1e-12, e.max()
    assert np.array_equal(R(gpu["iterations"]), R(ref["iterations"]))
    # ice-free cells keep the ocean temperature as interface temperature
    free = ~ice & (R(st.fields["inactive"]) == 0)
    assert np.allclose(R(gpu["interface_temperature"])[free], R(st.fields["T_oc"])[free], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", ["f32", "f32_adaptive"])
def test_atmosphere_sea_ice_f32_polish(oracle, precision):
    """FP32 sweep (skin temperature in delta form) + FP64 polish, and the adaptive mode that
    keeps the FP32 result of well-conditioned cells; both within 1e-5."""
    st = syn.coupled(seed=22, nx=120, ny=64, lat_s=-80, lat_n=80, land=0.0, interpolate=False)
    spec = P.atmosphere_sea_ice_interface_spec()
    ref = oracle.ai_fluxes(spec.to_c(), st.layout, widen(st.fields), st.fields["ice_temperature"])
    gpu = run_ai(spec, st, precision)
    R = st.layout.ring
    for k in F.AI_OUTPUTS:
        e = rel_err(R(gpu[k]), R(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-5, (k, e.max())
    e = rel_err(R(gpu["interface_temperature"]) + 273.15, R(ref["interface_temperature"]) + 273.15)
    assert e.max() <= 1e-5, e.max()


def test_sea_ice_ocean_fluxes_match_oracle(oracle, coupled64):
    import torch
    st = coupled64
    L = st.layout
    nz = 3
    T3 = np.stack([st.fields["T_oc"] - 0.2 * k for k in range(nz)])[::-1].copy()   # level nz is the top
    S3 = np.stack([st.fields["S_oc"] + 0.1 * k for k in range(nz)])[::-1].copy()
    dz = np.array([40.0, 20.0, 10.0])
    spec = P.SeaIceOceanSpec()
    inputs = dict(ice_salinity=st.fields["ice_salinity"], ice_thickness=st.fields["ice_thickness"],
                  consolidation_thickness=st.fields["consolidation_thickness"],
                  ice_concentration=st.fields["ice_concentration"], internal_temperature=st.fields["ice_temperature"],
                  ice_mass_flux=st.fields["ice_mass_flux"], snow_mass_flux=st.fields["snow_mass_flux"])
    ref = oracle.io_fluxes(spec.to_c(nz=nz, stride_k=L.shape[0] * L.shape[1]), L, inputs, T3, S3, dz)
    dev = api.to_device(inputs)
    out = {k: torch.zeros(L.shape, dtype=torch.float64, device="cuda") for k in F.IO_OUTPUTS}
    T3d = torch.from_numpy(T3).cuda()
    api.compute_sea_ice_ocean_fluxes(spec, L, dev, out, T3d, torch.from_numpy(S3).cuda(),
                                     torch.from_numpy(dz).cuda())
    torch.cuda.synchronize()
    I = L.interior
    for k in F.IO_OUTPUTS:
        e = rel_err(I(to_numpy(out[k])), I(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-12, (k, e.max())
    assert np.array_equal(to_numpy(T3d), ref["T_oc"])
    assert (I(ref["frazil_heat"]) < 0).any()   # some supercooled cells formed frazil


def test_sea_ice_ocean_fluxes_fp32_fields(oracle, coupled64):
    """FP32 fields: the sea-ice-ocean fluxes against the FP64 oracle on the same FP32
    inputs. The interface heat q = eta (T_N - T_b) + kappa (T_i - T_b) cancels where the
    ocean is near its melting point, so under ice the kernel solves the interface
    conditions in FP64 from the FP32 inputs: the interface heat, temperature and salinity
    of ice-covered cells are within 1e-6 relative of the oracle (FP32's final rounding).
    The other outputs are computed in FP32 (the reference's Float32 kernel): within
    1e-5 of each output's largest magnitude, 1e-5 relative on 99 % of the cells; the
    frazil-adjusted temperatures within 1e-6 K."""
    import torch
    st = coupled64
    L = st.layout
    nz = 3
    f32 = lambda x: np.asarray(x, dtype=np.float32)
    T3 = f32(np.stack([st.fields["T_oc"] - 0.2 * k for k in range(nz)])[::-1])
    S3 = f32(np.stack([st.fields["S_oc"] + 0.1 * k for k in range(nz)])[::-1])
    dz = np.array([40.0, 20.0, 10.0])
    spec = P.SeaIceOceanSpec()
    inputs = {k: f32(st.fields[v]) for k, v in dict(
        ice_salinity="ice_salinity", ice_thickness="ice_thickness", consolidation_thickness="consolidation_thickness",
        ice_concentration="ice_concentration", internal_temperature="ice_temperature",
        ice_mass_flux="ice_mass_flux", snow_mass_flux="snow_mass_flux").items()}
    ref = oracle.io_fluxes(spec.to_c(nz=nz, stride_k=L.shape[0] * L.shape[1]), L, widen(inputs),
                           T3.astype(np.float64), S3.astype(np.float64), dz)
    dev = api.to_device(inputs)
    out = {k: torch.zeros(L.shape, dtype=torch.float32, device="cuda") for k in F.IO_OUTPUTS}
    T3d = torch.from_numpy(np.ascontiguousarray(T3)).cuda()
    api.compute_sea_ice_ocean_fluxes(spec, L, dev, out, T3d, torch.from_numpy(np.ascontiguousarray(S3)).cuda(),
                                     torch.from_numpy(dz).cuda())
    torch.cuda.synchronize()
    I = L.interior
    ice = I(inputs["ice_concentration"]) > 0
    assert ice.sum() > 1000
    for k in F.IO_OUTPUTS:
        g, r = I(to_numpy(out[k])).astype(np.float64), I(ref[k])
        assert np.abs(g - r).max() <= 1e-5 * np.abs(r).max(), k
        assert np.percentile(rel_err(g, r, floor_frac=1e-6), 99) <= 1e-5, k
        if k in ("interface_heat", "interface_T", "interface_S"):
            e = rel_err(g[ice], r[ice], floor_frac=1e-6)
            assert e.max() <= 1e-6, (k, float(e.max()))
    assert np.abs(to_numpy(T3d).astype(np.float64) - ref["T_oc"]).max() <= 1e-6


def test_interpolation_matches_oracle(oracle):
    import torch
    st = syn.ao_quarter_land(nx=200, ny=80, dtype=np.float64)
    at = st.atmos
    ag = api.atmos_grid_struct(at)
    coords = api.exchange_coords(st.coords)
    ref = oracle.interpolate(st.layout, coords, ag, at["arrays"], at["time_weight"])
    src = api.to_device(at["arrays"])
    out = {n: torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda") for n in src}
    api.interpolate_atmosphere_state(st.layout, st.coords, at, src, out, at["time_weight"])
    fi = torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda")
    fj = torch.zeros_like(fi)
    api.compute_fractional_indices(st.layout, st.coords, at, fi, fj)
    out2 = {n: torch.zeros_like(out[n]) for n in src}
    api.interpolate_atmosphere_state(st.layout, st.coords, at, src, out2, at["time_weight"], frac=(fi, fj))
    torch.cuda.synchronize()
    R = st.layout.ring
    for n in src:
        assert rel_err(R(to_numpy(out[n])), R(ref[n]), floor_frac=1e-6).max() <= 1e-13, n
        assert np.array_equal(to_numpy(out[n]), to_numpy(out2[n])), n


@pytest.mark.parametrize("nx,ny,lon_w,lon_e,lat_s,lat_n,dtype", [
    (720, 96, -10.0, 350.0, -70.0, 70.0, np.float64),    # longitudes across the periodic seam
    (300, 70, 0.0, 360.0, 80.0, -80.0, np.float64),      # latitude decreasing with j
    (1440, 40, 0.0, 360.0, -70.0, 70.0, np.float32),     # quarter degree, FP32 fields
    (100, 50, 0.0, 360.0, -80.0, 80.0, np.float64),      # coarser than the atmosphere (gather kernel)
    (37, 5, 33.0, 47.0, 61.0, 62.0, np.float64),         # one partial tile
])
def test_interpolation_tiles_match_the_gather_kernel(oracle, nx, ny, lon_w, lon_e, lat_s, lat_n, dtype):
    """On a regular grid without caches the interpolation stages each tile's coarse stencil in
    shared memory (or, when the footprint is too large, gathers per cell): bit-identical to the
    gather kernel reading the fractional-index caches, and to the oracle to 1e-13 (FP64)."""
    import torch
    st = syn.ao_quarter_land(nx=nx, ny=ny, dtype=dtype)
    c = syn.lonlat(nx, ny, lat_s, lat_n, lon_w, lon_e)
    at = st.atmos
    src = api.to_device(at["arrays"])
    tdt = src["T"].dtype
    out = {n: torch.full(st.layout.shape, float("nan"), dtype=tdt, device="cuda") for n in src}
    api.interpolate_atmosphere_state(st.layout, c, at, src, out, at["time_weight"])
    fi = torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda")
    fj = torch.zeros_like(fi)
    api.compute_fractional_indices(st.layout, c, at, fi, fj)
    out2 = {n: torch.full_like(out[n], float("nan")) for n in src}
    api.interpolate_atmosphere_state(st.layout, c, at, src, out2, at["time_weight"], frac=(fi, fj))
    torch.cuda.synchronize()
    R = st.layout.ring
    for n in src:
        assert np.array_equal(R(to_numpy(out[n])), R(to_numpy(out2[n]))), n
    if dtype == np.float64:
        ref = oracle.interpolate(st.layout, api.exchange_coords(c), api.atmos_grid_struct(at), at["arrays"],
                                 at["time_weight"])
        for n in src:
            assert rel_err(R(to_numpy(out[n])), R(ref[n]), floor_frac=1e-6).max() <= 1e-13, n


def test_interpolation_fp32_fields(oracle):
    """FP32 fields interpolate in FP32 arithmetic, like the reference's Float32 kernels: against
    the FP64 oracle on the same (FP32) atmosphere, positive fields (T, p, q, radiation) are within
    1e-6 relative and every field within 1e-6 of its largest magnitude (u and v change sign, so
    their bilinear sums can cancel)."""
    import torch
    st = syn.ao_quarter_land(nx=200, ny=80, dtype=np.float32)
    at = st.atmos
    ag = api.atmos_grid_struct(at)
    coords = api.exchange_coords(st.coords)
    ref = oracle.interpolate(st.layout, coords, ag, widen(at["arrays"]), at["time_weight"])
    src = api.to_device(at["arrays"])
    assert src["T"].dtype == torch.float32
    out = {n: torch.zeros(st.layout.shape, dtype=torch.float32, device="cuda") for n in src}
    api.interpolate_atmosphere_state(st.layout, st.coords, at, src, out, at["time_weight"])
    torch.cuda.synchronize()
    R = st.layout.ring
    for n in src:
        g, r = R(to_numpy(out[n])).astype(np.float64), R(ref[n])
        assert np.abs(g - r).max() <= 1e-6 * np.abs(r).max(), n
        if n in ("T", "p", "q", "sw", "lw"):
            assert rel_err(g, r, floor_frac=1e-6).max() <= 1e-6, n


def test_assembly_fp32_fields(oracle, coupled64):
    """FP32 fields assemble in FP32 arithmetic: within 1e-6 of each output's largest magnitude,
    and 1e-5 relative on 99 % of the cells. The net heat flux sums terms of opposite sign
    (emitted longwave ~400 W/m2 against absorbed longwave and the turbulent fluxes), so the
    FP32 rounding of the terms is a larger fraction of the sum."""
    import torch
    st = coupled64
    L = st.layout
    rng = np.random.default_rng(5)
    f32 = lambda a: np.asarray(a, dtype=np.float32)
    names_in = ["ao_sensible", "ao_latent", "ao_water_vapor", "ao_x_momentum", "ao_y_momentum",
                "io_interface_heat", "io_frazil_heat", "io_salt", "io_freshwater", "io_x_momentum",
                "io_y_momentum", "ai_sensible", "ai_latent", "ai_x_momentum", "ai_y_momentum", "intercepted_snow"]
    arrays = {n: f32(rng.normal(0, 50, L.shape)) for n in names_in}
    arrays["ao_interface_temperature"] = f32(st.fields["T_oc"])
    arrays["ai_interface_temperature"] = f32(st.fields["ice_temperature"])
    arrays.update(ice_concentration=f32(st.fields["ice_concentration"]), ocean_surface_temperature=f32(st.fields["T_oc"]),
                  rain=f32(st.fields["rain"]), snow=f32(st.fields["snow"]), sw_down=f32(st.fields["sw_down"]),
                  lw_down=f32(st.fields["lw_down"]), inactive=st.fields["inactive"])
    outs = ["ocean_u", "ocean_v", "ocean_T", "ocean_S", "ocean_eta", "ocean_heat_content", "ice_top_heat",
            "ice_top_snowfall", "ice_top_u", "ice_top_v", "ice_bottom_heat", "ocean_upwelling_longwave",
            "ocean_downwelling_longwave", "ocean_downwelling_shortwave", "ice_upwelling_longwave",
            "ice_downwelling_longwave", "ice_downwelling_shortwave"]
    host = widen(arrays)
    host.update({n: np.zeros(L.shape) for n in outs})
    spec = P.AssemblySpec()
    pc = spec.to_c()
    for which in ("ocean", "sea_ice", "ocean_radiation", "sea_ice_radiation"):
        oracle.assemble(pc, L, host, which)
    dev = api.to_device(arrays)
    dev.update({n: torch.zeros(L.shape, dtype=torch.float32, device="cuda") for n in outs})
    api.assemble_net_ocean_fluxes(spec, L, dev)
    api.assemble_net_sea_ice_fluxes(spec, L, dev)
    api.apply_air_sea_radiative_fluxes(spec, L, dev)
    api.apply_air_sea_ice_radiative_fluxes(spec, L, dev)
    torch.cuda.synchronize()
    I = L.interior
    for n in outs:
        g, r = I(to_numpy(dev[n])).astype(np.float64), I(host[n])
        assert np.abs(g - r).max() <= 1e-6 * np.abs(r).max(), n
        assert np.percentile(rel_err(g, r, floor_frac=1e-6), 99) <= 1e-5, n


def test_assembly_and_radiation_match_oracle(oracle, coupled64):
    import torch
    st = coupled64
    L = st.layout
    rng = np.random.default_rng(4)
    names_in = ["ao_sensible", "ao_latent", "ao_water_vapor", "ao_x_momentum", "ao_y_momentum",
                "ao_interface_temperature", "io_interface_heat", "io_frazil_heat", "io_salt", "io_freshwater",
                "io_x_momentum", "io_y_momentum", "ai_sensible", "ai_latent", "ai_x_momentum", "ai_y_momentum",
                "ai_interface_temperature", "intercepted_snow"]
    arrays = {n: rng.normal(0, 50, L.shape) for n in names_in}
    arrays["ao_interface_temperature"] = st.fields["T_oc"].copy()
    arrays["ai_interface_temperature"] = st.fields["ice_temperature"].copy()
    arrays.update(ice_concentration=st.fields["ice_concentration"], ocean_surface_temperature=st.fields["T_oc"],
                  rain=st.fields["rain"], snow=st.fields["snow"], sw_down=st.fields["sw_down"],
                  lw_down=st.fields["lw_down"], inactive=st.fields["inactive"])
    outs = ["ocean_u", "ocean_v", "ocean_T", "ocean_S", "ocean_eta", "ocean_heat_content", "ice_top_heat",
            "ice_top_snowfall", "ice_top_u", "ice_top_v", "ice_bottom_heat", "ocean_upwelling_longwave",
            "ocean_downwelling_longwave", "ocean_downwelling_shortwave", "ice_upwelling_longwave",
            "ice_downwelling_longwave", "ice_downwelling_shortwave"]
    host = dict(arrays)
    host.update({n: np.zeros(L.shape) for n in outs})
    spec = P.AssemblySpec()
    pc = spec.to_c()
    for which in ("ocean", "sea_ice", "ocean_radiation", "sea_ice_radiation"):
        oracle.assemble(pc, L, host, which)
    dev = api.to_device(arrays)
    dev.update({n: torch.zeros(L.shape, dtype=torch.float64, device="cuda") for n in outs})
    api.assemble_net_ocean_fluxes(spec, L, dev)
    api.assemble_net_sea_ice_fluxes(spec, L, dev)
    api.apply_air_sea_radiative_fluxes(spec, L, dev)
    api.apply_air_sea_ice_radiative_fluxes(spec, L, dev)
    torch.cuda.synchronize()
    I = L.interior
    for n in outs:
        e = rel_err(I(to_numpy(dev[n])), I(host[n]), floor_frac=1e-6)
        assert e.max() <= 1e-12, (n, e.max())
    land = I(st.fields["inactive"]) != 0
    assert np.all(I(to_numpy(dev["ocean_T"]))[land] == 0)


@pytest.mark.parametrize("wind", [0.0, 0.7, 1000.0])
def test_sea_ice_calm_cells_replay_from_the_classify_pass(oracle, coupled64, wind):
    """The adaptive sea-ice solve sends the cells whose wind is below calm_replay_wind from its
    classify pass straight to the reference's FP64 iteration, on a stream of their own beside
    pass 1: none (0, the default), the calm ones (0.7 m/s) or every ice cell (1000 m/s). The
    fluxes stay within 1e-5 of the oracle, every cell is counted once, and with every cell
    replayed all of them are solved by the FP64 iteration."""
    import torch
    st = coupled64
    spec = P.atmosphere_sea_ice_interface_spec()
    ref = oracle.ai_fluxes(spec.to_c(), st.layout, st.fields, st.fields["ice_temperature"])
    dev = api.to_device({k: st.fields.get(k) for k in F.AI_INPUTS if k in st.fields})
    out = {k: torch.zeros(st.layout.shape, dtype=torch.float64, device="cuda") for k in F.AI_OUTPUTS}
    out["interface_temperature"] = torch.from_numpy(st.fields["ice_temperature"].copy()).cuda()
    s = api.compute_atmosphere_sea_ice_fluxes(spec, st.layout, dev, out, precision="f32_adaptive", stats=True,
                                              calm_replay_wind=wind)
    torch.cuda.synchronize()
    R = st.layout.ring
    conv = R(ref["iterations"]) < 100
    for k in F.AI_OUTPUTS + ("interface_temperature",):
        g, r = R(to_numpy(out[k])), R(ref[k])
        if k == "interface_temperature":
            g, r = g + 273.15, r + 273.15
        e = rel_err(g, r, floor_frac=1e-6)[conv]
        assert e.max() <= 1e-5, (wind, k, float(e.max()))
    ice = int(((R(st.fields["ice_concentration"]) > 0) & (R(st.fields["inactive"]) == 0)).sum())
    assert s["cells"] == R(st.fields["ice_concentration"]).size
    assert s["solved"] == ice
    if wind > 100:
        assert s["fp64_redo"] == ice and s["polished"] == 0


def test_ensemble_members_use_their_own_parameters(oracle):
    import torch
    members = 4
    st = syn.ensemble(seed=9, members=members, nx=48, ny=24)
    specs = []
    for pert in st.perturbations:
        mom = P.MomentumRoughnessLength(wave_formulation=pert["charnock"],
                                        smooth_wall_parameter=0.11 * pert["nu_scale"])
        sc = P.ScalarRoughnessLength(reynolds_number_scaling_function=P.ReynoldsScalingFunction(
            5.85e-5 * pert["A_scale"], 0.72 * pert["b_scale"]))
        flux = P.SimilarityTheoryFluxes(subgrid_velocities=P.ConvectiveGustiness(1.2, pert["minimum_gustiness"]),
                                        momentum_roughness_length=mom, temperature_roughness_length=sc,
                                        water_vapor_roughness_length=sc)
        specs.append(P.atmosphere_ocean_interface_spec(flux_formulation=flux))
    dev = api.to_device({k: st.fields[k] for k in F.AO_INPUTS if k in st.fields})
    out = {k: torch.zeros((members,) + st.layout.shape, dtype=torch.float32, device="cuda") for k in F.AO_OUTPUTS}
    for prec in ("f64", "f32"):
        api.compute_atmosphere_ocean_fluxes_ensemble(specs, st.layout, dev, out, precision=prec)
        torch.cuda.synchronize()
        for m in range(members):
            fm = {k: st.fields[k][m] for k in st.fields}
            ref = oracle.ao_fluxes(specs[m].to_c(), st.layout, widen(fm))
            for k in ("latent_heat", "sensible_heat", "x_momentum", "friction_velocity"):
                g = st.layout.ring(to_numpy(out[k][m]))
                e = rel_err(g, st.layout.ring(ref[k]), floor_frac=1e-6)
                assert e.max() <= (1e-6 if prec == "f64" else 1e-5), (prec, m, k, e.max())
