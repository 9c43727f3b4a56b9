"""The coupling-step state and `update_state` (time_step_earth_system_model.jl:38-83).

`CoupledModel` holds, on one device, what `update_state!(::EarthSystemModel)`
touches for an ocean + sea-ice model forced by a PrescribedAtmosphere and
PrescribedRadiation: the coarse atmosphere snapshots, the exchange-grid state,
the interface fluxes and the net boundary fluxes. `update_state` runs the four
phases through libnesf.so:
  1. interpolate_state!        atmosphere + radiation onto the exchange grid
  2. compute_*_fluxes!         atmosphere-ocean, atmosphere-sea-ice, sea-ice-ocean
  3. update_net_fluxes!        ocean and sea ice
  4. apply_*_radiative_fluxes! ocean and sea ice
"""
import numpy as np

from . import api
from . import fields as F
from . import params as P

OCEAN_NET = ("ocean_u", "ocean_v", "ocean_T", "ocean_S", "ocean_eta", "ocean_heat_content")
ICE_NET = ("ice_top_heat", "ice_top_snowfall", "ice_top_u", "ice_top_v", "ice_bottom_heat")
RAD_DIAG = ("ocean_upwelling_longwave", "ocean_downwelling_longwave", "ocean_downwelling_shortwave",
            "ice_upwelling_longwave", "ice_downwelling_longwave", "ice_downwelling_shortwave")
ATMOS_NAMES = ("u", "v", "T", "q", "p", "rain", "snow", "sw", "lw")
EXCHANGE_ATMOS = {"u": "u_atm", "v": "v_atm", "T": "T_atm", "q": "q_atm", "p": "p_atm", "rain": "rain",
                  "snow": "snow", "sw": "sw_down", "lw": "lw_down"}
# per-step host inputs of the end-to-end path (everything a coupling step consumes)
STEP_INPUTS = ("u_oc", "v_oc", "T_oc", "S_oc", "ice_concentration", "ice_thickness", "snow_thickness",
               "consolidation_thickness", "ice_salinity", "ice_temperature", "ice_mass_flux", "snow_mass_flux")


class CoupledModel:
    def __init__(self, state, device="cuda", ao_spec=None, ai_spec=None, io_spec=None, assembly_spec=None,
                 dz_top=10.0):
        import torch
        self.torch = torch
        self.state = state
        self.layout = state.layout
        self.coords = state.coords
        self.device = device
        L = self.layout
        f = state.fields
        self.dtype = torch.float32 if state.dtype == np.float32 else torch.float64
        dt = self.dtype
        self.ao_spec = ao_spec or P.atmosphere_ocean_interface_spec()
        self.ai_spec = ai_spec or P.atmosphere_sea_ice_interface_spec()
        self.io_spec = io_spec or P.SeaIceOceanSpec()
        self.asm_spec = assembly_spec or P.AssemblySpec()
        z = lambda: torch.zeros(L.shape, dtype=dt, device=device)
        # exchange-grid surface state
        self.x = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in f.items()}
        self.T3 = self.x["T_oc"].view((1,) + L.shape)
        self.S3 = self.x["S_oc"].view((1,) + L.shape)
        self.dz = torch.tensor([dz_top], dtype=torch.float64, device=device)
        self.atmos = state.atmos
        if state.atmos is not None:
            self.atmos_src = {n: torch.from_numpy(state.atmos["arrays"][n]).to(device) for n in ATMOS_NAMES}
            for n in ATMOS_NAMES:
                self.x[EXCHANGE_ATMOS[n]] = z()
            # initialize!(exchanger) computes the fractional indices once
            # (prescribed_atmosphere_regridder.jl:41-49). On this regular longitude-latitude exchange
            # grid they depend on the column and on the row alone, so the interpolation computes them
            # per tile from the coordinates (the same values) instead of reading two FP64 caches per
            # cell; `fractional_indices()` computes the caches for a caller that wants them.
            self.fi = self.fj = None
        self.ai_T = self.x["ice_temperature"].clone()     # AI interface (top surface) temperature, in/out
        self.ao = {k: z() for k in F.AO_OUTPUTS}
        self.ai = {k: z() for k in F.AI_OUTPUTS}
        self.ai["interface_temperature"] = self.ai_T
        self.io = {k: z() for k in F.IO_OUTPUTS}
        self.net = {k: z() for k in OCEAN_NET + ICE_NET + RAD_DIAG}
        self.zero_io_stress = z()
        self.intercepted = z()
        self.mlp = None       # a trained warm.WarmStartNetwork: warm start of the FP32 solvers
        self.iterations = None   # {"ao": int32 tensor, "ai": ...} to record per-cell iteration counts

    # -------------------------------------------------------------- phases
    def interpolate_state(self, stream=None):
        if self.atmos is None:
            return 0
        out = {n: self.x[EXCHANGE_ATMOS[n]] for n in ATMOS_NAMES}
        api.interpolate_atmosphere_state(self.layout, self.coords, self.atmos, self.atmos_src, out,
                                         self.atmos["time_weight"], stream=stream)
        return 1

    def fractional_indices(self):
        """The exchanger's fractional-index fields (nesf_compute_fractional_indices), FP64 on the
        device: what initialize!(exchanger) stores."""
        torch = self.torch
        fi = torch.zeros(self.layout.shape, dtype=torch.float64, device=self.device)
        fj = torch.zeros_like(fi)
        api.compute_fractional_indices(self.layout, self.coords, self.atmos, fi, fj)
        return fi, fj

    def compute_fluxes(self, precision="f64", polish_maxiter=0, stats=False, stream=None):
        x = self.x
        s_ao = api.compute_atmosphere_ocean_fluxes(self.ao_spec, self.layout, x, self.ao, precision=precision,
                                                   polish_maxiter=polish_maxiter, stats=stats, stream=stream,
                                                   mlp=self.mlp,
                                                   iterations=self.iterations["ao"] if self.iterations else None)
        ai_state = {k: x.get(k) for k in F.AI_INPUTS}
        s_ai = api.compute_atmosphere_sea_ice_fluxes(self.ai_spec, self.layout, ai_state, self.ai,
                                                     precision=precision, polish_maxiter=polish_maxiter,
                                                     stats=stats, stream=stream, mlp=self.mlp,
                                                     iterations=self.iterations["ai"] if self.iterations else None)
        io_state = {"ice_salinity": x["ice_salinity"], "ice_thickness": x["ice_thickness"],
                    "consolidation_thickness": x["consolidation_thickness"],
                    "ice_concentration": x["ice_concentration"], "internal_temperature": x["ice_temperature"],
                    "ice_mass_flux": x["ice_mass_flux"], "snow_mass_flux": x["snow_mass_flux"]}
        api.compute_sea_ice_ocean_fluxes(self.io_spec, self.layout, io_state, self.io, self.T3, self.S3, self.dz,
                                         stream=stream)
        return (s_ao, s_ai) if stats else 3

    def assembly_arrays(self):
        x, ao, ai, io, n = self.x, self.ao, self.ai, self.io, self.net
        arr = dict(inactive=x["inactive"], ice_concentration=x["ice_concentration"],
                   ocean_surface_temperature=x["T_oc"], rain=x["rain"], snow=x["snow"],
                   intercepted_snow=self.intercepted, ao_sensible=ao["sensible_heat"], ao_latent=ao["latent_heat"],
                   ao_water_vapor=ao["water_vapor"], ao_x_momentum=ao["x_momentum"], ao_y_momentum=ao["y_momentum"],
                   ao_interface_temperature=ao["interface_temperature"], io_interface_heat=io["interface_heat"],
                   io_frazil_heat=io["frazil_heat"], io_salt=io["salt"], io_freshwater=io["freshwater"],
                   io_x_momentum=self.zero_io_stress, io_y_momentum=self.zero_io_stress,
                   ai_sensible=ai["sensible_heat"], ai_latent=ai["latent_heat"], ai_x_momentum=ai["x_momentum"],
                   ai_y_momentum=ai["y_momentum"], ai_interface_temperature=ai["interface_temperature"],
                   sw_down=x["sw_down"], lw_down=x["lw_down"])
        arr.update(n)
        return arr

    def update_net_fluxes(self, stream=None):
        arr = self.assembly_arrays()
        api.assemble_net_ocean_fluxes(self.asm_spec, self.layout, arr, stream=stream)
        api.assemble_net_sea_ice_fluxes(self.asm_spec, self.layout, arr, stream=stream)
        api.apply_air_sea_radiative_fluxes(self.asm_spec, self.layout, arr, stream=stream)
        api.apply_air_sea_ice_radiative_fluxes(self.asm_spec, self.layout, arr, stream=stream)
        return 4

    def update_state(self, precision="f64", polish_maxiter=0, stream=None):
        """One coupling step through the per-phase entry points; returns the number of
        kernels it launches."""
        self.interpolate_state(stream)
        self.compute_fluxes(precision, polish_maxiter, stream=stream)
        self.update_net_fluxes(stream)
        return self.kernels_per_step(precision)

    def kernels_per_step(self, precision, native=False):
        """Kernels one step launches: interpolation; per solve classify + solve (+ the packed
        polish pass of the adaptive mode, + the replay passes of the FP32 modes: the adaptive
        mode replays pass 1's cells beside the polish pass and the polish pass's after it);
        the ocean's warm-start inference; sea-ice-ocean (in the native step its fluxes and its
        frazil adjustment apart); ocean and sea-ice assembly with their radiative add-ons (in
        the native step inside the assembly kernels)."""
        fast = precision != "f64" and precision != "plain"
        adaptive = precision == "f32_adaptive"
        per_solve = 2 + adaptive + (2 if adaptive else 1) * fast
        warm = 1 if fast and self.mlp is not None else 0
        return ((1 if self.atmos is not None else 0) + 2 * per_solve + warm + (2 if native else 1) +
                (2 if native else 4))

    # ------------------------------------------------- native step and graph
    def step_args(self):
        """nesf_coupling_step arguments over this model's tensors (built once)."""
        if getattr(self, "_step", None) is None:
            x = self.x
            ao_arrays = {k: x.get(k) for k in F.AO_INPUTS}
            ao_arrays.update({k: self.ao.get(k) for k in F.AO_OUTPUTS})
            ai_arrays = {k: x.get(k) for k in F.AI_INPUTS}
            ai_arrays.update({k: self.ai.get(k) for k in F.AI_OUTPUTS})
            ai_arrays["interface_temperature"] = self.ai["interface_temperature"]
            io_arrays = {"ice_salinity": x["ice_salinity"], "ice_thickness": x["ice_thickness"],
                         "consolidation_thickness": x["consolidation_thickness"],
                         "ice_concentration": x["ice_concentration"], "internal_temperature": x["ice_temperature"],
                         "ice_mass_flux": x["ice_mass_flux"], "snow_mass_flux": x["snow_mass_flux"]}
            io_arrays.update({k: self.io.get(k) for k in F.IO_OUTPUTS})
            io_arrays.update(T_oc=self.T3, S_oc=self.S3, dz=self.dz)
            interp = None
            if self.atmos is not None:
                out = {n: self.x[EXCHANGE_ATMOS[n]] for n in ATMOS_NAMES}
                interp = (self.coords, self.atmos, self.atmos_src, out, None, self.atmos["time_weight"])
            L = self.layout
            self._step = api.CouplingStep(self.ao_spec, L, ao_arrays, self.ai_spec, ai_arrays, self.io_spec,
                                          io_arrays, (self.T3.shape[0], L.shape[0] * L.shape[1]), interp,
                                          self.asm_spec, self.assembly_arrays(), radiation=True)
        return self._step

    def native_step(self, precision="f32_adaptive", stream=None):
        """One coupling step through nesf_coupling_step; returns the kernels launched."""
        api.coupling_step(self.step_args(), precision, stream=stream, mlp=self.mlp)
        return self.kernels_per_step(precision, native=True)

    def autotune(self, precision="f32_adaptive", reps=5, cache=None):
        """Tune the default context's launch shapes and schedule on this model's step
        (nesf_autotune; through the tuning-cache file `cache` when given). The steps run for
        real; the state is reset afterwards."""
        t = api.autotune(self.step_args(), precision, reps=reps, mlp=self.mlp, cache=cache)
        self.reset()
        return t

    def capture(self, precision="f32_adaptive", calm_replay_wind=None):
        """Capture one coupling step as a CUDA graph (nesf_graph_capture); `calm_replay_wind`
        overrides the library's default for the sea-ice solve's calm cells."""
        self.graph = api.Graph(self.step_args(), precision, mlp=self.mlp, calm_replay_wind=calm_replay_wind)
        self.graph_precision = precision
        return self.graph

    def graph_step(self, stream=None, time_weight=None):
        """Replay the captured step; returns the kernels it runs."""
        if time_weight is not None:
            self.graph.set_time_weight(time_weight)
        self.graph.launch(stream)
        return self.kernels_per_step(self.graph_precision, native=True)

    # ------------------------------------------------------ conservation
    def row_areas(self, radius=6.371e6):
        """Cell areas of the regular longitude-latitude exchange grid by row j = 1..ny
        (R^2 dlambda (sin phi_north - sin phi_south)), FP64 on the device."""
        c, L = self.coords, self.layout
        lat = c.lat0 + np.arange(L.ny) * c.dlat
        s = np.sin(np.radians(lat + c.dlat / 2)) - np.sin(np.radians(lat - c.dlat / 2))
        a = radius ** 2 * np.radians(abs(c.dlon)) * np.abs(s)
        return self.torch.from_numpy(a).to(self.device)

    def heat_budget(self):
        """The ocean heat budget of the last assembled step as compensated FP64 area integrals:
        rho_o c_o int dA(J_T) against its sources, int dA(1 - aleph, Q_T + Q_v) + int dA(Q_io)
        + int dA(1 - aleph, I_up) - int dA(I_lw) - int dA(I_sw) (the absorbed radiation is
        assembled with its (1 - aleph) factor). Returns (rho_o c_o int J_T, sum of sources,
        relative residual)."""
        n, ao, io = self.net, self.ao, self.io
        open_water = 1 - self.x["ice_concentration"]
        rows = self.row_areas()
        fields = [n["ocean_T"], ao["sensible_heat"], ao["latent_heat"], io["interface_heat"],
                  n["ocean_upwelling_longwave"], n["ocean_downwelling_longwave"], n["ocean_downwelling_shortwave"]]
        factors = [None, open_water, open_water, None, open_water, None, None]
        r = api.area_integrals(self.layout, fields, factors, inactive=self.x["inactive"], row_area=rows)
        v = r.cpu().numpy()
        tot = v[:, 0] + v[:, 1]
        rc = self.asm_spec.ocean_reference_density * self.asm_spec.ocean_heat_capacity
        lhs = rc * tot[0]
        terms = np.array([tot[1], tot[2], tot[3], tot[4], -tot[5], -tot[6]])
        rhs = float(np.sum(terms))
        return lhs, rhs, abs(lhs - rhs) / max(abs(lhs), float(np.abs(terms).sum()))

    # ---------------------------------------------------------- bookkeeping
    def active_cells(self):
        """Cells solved per step: water cells (atmosphere-ocean) + ice-covered water cells
        (atmosphere-sea-ice), interior only."""
        L = self.layout
        water = L.interior(self.state.fields["inactive"]) == 0
        ice = L.interior(self.state.fields["ice_concentration"]) > 0
        return int(water.sum()), int((water & ice).sum())

    def reset(self):
        """Restore the state a step mutates (AI interface temperature, frazil-adjusted T)."""
        f = self.state.fields
        self.x["T_oc"].copy_(self.torch.from_numpy(f["T_oc"]).to(self.device))
        self.ai_T.copy_(self.x["ice_temperature"])
