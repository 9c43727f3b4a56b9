"""Benchmark of the interface-flux coupling step on one GB300 (or N independent replicas).

Workload: the 1/8 degree coupled ocean + sea-ice exchange grid (2880 x 1280,
latitude -80..80, 30 % land, sea ice poleward of 55 degrees), forced by a
640 x 320 prescribed atmosphere at two 3-hourly snapshots interpolated onto the
exchange grid; FP32 fields in HBM. One step = update_state: interpolation,
atmosphere-ocean + atmosphere-sea-ice + sea-ice-ocean fluxes, net ocean and
sea-ice flux assembly with radiation. The step's working set (~0.8 GB) exceeds
L2, so no flush is needed between timed steps.

Metric: flux cells/s (water cells solved at the atmosphere-ocean interface +
ice-covered cells at the atmosphere-sea-ice interface, per second), for the
FP32 + FP64-polish solver; the plain FP64 solver is timed on the same step and
reported beside it, with the max relative flux error of the fast solver.

--impl reference times the CPU restatement of the reference's path (the
reference is Julia; no Julia toolchain is available) on all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "numericalearth.jl_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "flux cells/s at <=1e-5 rel err: FP32+batch+warm-start vs plain FP64, 1 GB300"
WORKLOAD = "coupled_eighth: 2880x1280 ocean+sea-ice exchange grid, 30% land, 640x320x2 prescribed atmosphere"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nesf", choices=["nesf", "reference"])
    ap.add_argument("--precision", default="f32_adaptive", choices=["f32_adaptive", "f32", "f64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="small grid (profiling captures)")
    ap.add_argument("--no-plain", action="store_true", help="time only --precision (profiling captures)")
    ap.add_argument("--cold", action="store_true", help="no learned warm start")
    ap.add_argument("--warm-samples", default="1e7", choices=["1e7", "4e5"], help="warm-start training set")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (no nesf_autotune)")
    ap.add_argument("--no-configs", action="store_true", help="skip the measurements of configurations 0-3")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        hist = {}
        for v in sm:
            hist[str(int(v))] = hist.get(str(int(v)), 0) + 1
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "sm_mhz_histogram": hist,
                "power_w_median": float(np.median([float(r[3]) for r in rows if _num(r[3])]))
                if any(_num(r[3]) for r in rows) else None}


def _num(x):
    try:
        float(x)
        return True
    except ValueError:
        return False


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def make_state(small):
    from nesf import synthetic as syn
    if small:
        return syn.coupled(seed=1004, nx=720, ny=320, lat_s=-80, lat_n=80, land=0.3, interpolate=True)
    return syn.coupled_eighth()


# algorithmic bytes per cell of each phase for FP32 fields (element size 4 B):
#  atmosphere-ocean solve: 9 inputs (u, v, T, p, q atmosphere; u, v, T, S ocean) + mask (1 B)
#                          read, 9 outputs written                       -> 18*4 + 1 = 73 B
#  atmosphere-sea-ice:     12 inputs + mask read, 6 outputs (incl. T_s)   -> 18*4 + 1 = 73 B
#  sea-ice-ocean:          T, S, Si, h, hc, aleph, T_int, E_i, E_s read; T (frazil), 6 outputs -> 16*4 = 64 B
#  interpolation:          9 exchange-grid outputs (+ 2 FP64 fractional indices read) -> 9*4 + 16 = 52 B
#  assembly + radiation:   ocean 17 reads + 6 writes, ice 11 reads + 5 writes, radiation 6 diag writes
# DRAM bytes (read + write) per solved cell of one ao_adaptive_kernel launch: ncu
# dram__bytes_read.sum + dram__bytes_write.sum on the --small case (17,448,960 + 65,024 bytes for
# 162,402 cells), scaled to the workload's launch by its cells. Above the 73 algorithmic bytes:
# the 64-byte record of cancelling differences per cell that the classify pass writes and
# pass 1 reads (scratch, not an input of the operator)
AO_KERNEL_DRAM_BYTES_PER_CELL = 107.8


# warm-start training sets: "1e7" -- about 1e7 solver-generated samples, the scale the
# 1/8-degree workload's configuration names: two open-ocean states of 2880 x 1280 with 0-40 m/s
# winds and -15..+10 K air-sea differences (7.4 M cells) and four coupled 1440 x 720 states
# like the workload's (2.9 M water cells); "4e5" -- the small set (four 360 x 180 open-ocean
# states, three coupled 360 x 180 states)
WARM_SETS = {
    "1e7": dict(open_ocean=[(2880, 1280)] * 2, coupled=[(1440, 720)] * 4,
                schedule=((2, 2e-3), (1, 5e-4), (1, 1e-4)), batch=4096),
    "4e5": dict(open_ocean=[(360, 180)] * 4, coupled=[(360, 180)] * 3,
                schedule=((12, 2e-3), (8, 5e-4), (5, 1e-4)), batch=2048),
}


def train_warm_start(seed=0, samples="1e7"):
    """Train the warm-start network on solver-generated samples (open-ocean states with 0-40 m/s
    winds and -15..+10 K air-sea differences, and coupled states like the workload's), on the
    tensor cores; returns the network and a summary (sample count, epochs, losses, seconds
    for the samples and for the training)."""
    import torch
    from nesf import params as P
    from nesf import synthetic as syn
    from nesf import warm
    cfg = WARM_SETS[samples]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    spec = P.atmosphere_ocean_interface_spec()

    def states():
        for k, (nx, ny) in enumerate(cfg["open_ocean"]):
            yield syn.warm_training_state(seed=7000 + k, nx=nx, ny=ny)
        for k, (nx, ny) in enumerate(cfg["coupled"]):
            yield syn.coupled(seed=7100 + k, nx=nx, ny=ny, lat_s=-80, lat_n=80, land=0.3, interpolate=False)

    x, t = warm.training_set(spec, states(), shuffle_seed=seed + 11)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net = warm.WarmStartNetwork(seed=seed)
    net.fit_normalization(x, t)
    losses = []
    for epochs, lr in cfg["schedule"]:
        losses += net.train(x, t, epochs=epochs, batch=cfg["batch"], lr=lr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    n = int(x.shape[0])
    del x, t
    return net, {"samples": n, "set": samples, "epochs": len(losses), "batch": cfg["batch"],
                 "loss_first": losses[0], "loss_last": losses[-1], "seconds_samples": t1 - t0,
                 "seconds_training": t2 - t1, "seconds": t2 - t0}


def phase_times(model, precision, reps=3):
    """Per-phase device time (ms) with CUDA events on the launching stream."""
    import torch
    s = torch.cuda.current_stream()
    names = ["interp", "ao", "ai", "io", "asm"]
    acc = {n: 0.0 for n in names}
    from nesf import api
    from nesf import fields as F
    for _ in range(reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        ev[0].record(s)
        model.interpolate_state()
        ev[1].record(s)
        api.compute_atmosphere_ocean_fluxes(model.ao_spec, model.layout, model.x, model.ao, precision=precision)
        ev[2].record(s)
        api.compute_atmosphere_sea_ice_fluxes(model.ai_spec, model.layout, {k: model.x.get(k) for k in F.AI_INPUTS},
                                              model.ai, precision=precision)
        ev[3].record(s)
        x = model.x
        api.compute_sea_ice_ocean_fluxes(model.io_spec, model.layout,
                                         {"ice_salinity": x["ice_salinity"], "ice_thickness": x["ice_thickness"],
                                          "consolidation_thickness": x["consolidation_thickness"],
                                          "ice_concentration": x["ice_concentration"],
                                          "internal_temperature": x["ice_temperature"],
                                          "ice_mass_flux": x["ice_mass_flux"], "snow_mass_flux": x["snow_mass_flux"]},
                                         model.io, model.T3, model.S3, model.dz)
        ev[4].record(s)
        model.update_net_fluxes()
        ev[5].record(s)
        torch.cuda.synchronize()
        for k, n in enumerate(names):
            acc[n] += ev[k].elapsed_time(ev[k + 1]) / reps
    return acc


REPEAT_ROUNDS = 5

# ncu pipe utilisation of the two pass-1 solve kernels (--set full, one launch each on the
# 720 x 320 coupled case): the profile summary named here holds the command and the figures.
NCU_PIPES = {
    "source": "profiles/solve_kernels_f32adaptive_coupled_720x320.md",
    "ao_adaptive_kernel": {"issue_active": 0.546, "fma_pipe": 0.211, "alu_pipe": 0.288, "xu_inst": 0.117,
                           "fp64_pipe": 0.019, "warps_active": 0.315, "lanes_active_per_warp_instruction": 24.1},
    "ai_adaptive_kernel": {"issue_active": 0.373, "fma_pipe": 0.122, "alu_pipe": 0.182, "xu_inst": 0.072,
                           "fp64_pipe": 0.009, "warps_active": 0.132, "lanes_active_per_warp_instruction": 18.8},
    "ai_replay_kernel_double_float": {"issue_active": 0.274, "fma_pipe": 0.192, "alu_pipe": 0.051, "xu_inst": 0.006,
                                      "fp64_pipe": 0.0, "warps_active": 0.058,
                                      "lanes_active_per_warp_instruction": 22.4},
}


def compute_roofline(work_t, work_f, t_ms, fp64_iters, clk):
    """The compute side of the main solve kernel's roofline: the work table's rates
    (NESF_WORK_*: transcendentals and flops of the reference's FP64 cold-start iterations)
    against peaks DERIVED from the SM count and the sampled SM clock (FP32: 128 lanes x 2
    flops per SM per cycle; MUFU: 16 per SM per cycle), beside the ncu pipe fractions."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * mhz * 1e6
    mufu_peak = sms * 16 * mhz * 1e6
    sec = t_ms / 1000.0 if t_ms else None
    flops = work_f / sec if sec else None
    trans = work_t / sec if sec else None
    return {"work_transcendentals": work_t, "work_flops": work_f, "transcendentals_per_s": trans,
            "flops_per_s": flops, "fp64_cold_start_iterations": fp64_iters,
            "fp32_peak_flops_derived": fp32_peak, "mufu_peak_ops_derived": mufu_peak,
            "frac_fp32_work_table": flops / fp32_peak if flops else None,
            "frac_mufu_work_table": trans / mufu_peak if trans else None,
            "peak_note": f"derived: {sms} SMs x 128 FP32 lanes x 2 flops (FMA) x {mhz:.0f} MHz; MUFU 16 / SM / "
                         "cycle. The work table counts the reference's FP64 cold-start iterations, so a "
                         "fraction above the pipes' own ncu fractions means iterations saved.",
            "ncu_pipes": NCU_PIPES}


def replay_round(model, steps, world):
    """One more timed round of `steps` replays of the captured step (already warm)."""
    import torch
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        model.graph_step()
    e1.record(s)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms


def time_steps(model, precision, steps, warmup, world):
    """Device time per coupling step, replaying the step captured as a CUDA graph."""
    import torch
    model.capture(precision)
    for _ in range(warmup):
        model.graph_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    e0.record(s)
    for _ in range(steps):
        launches += model.graph_step()
    e1.record(s)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, launches


def step_timeline(model, precision):
    """Kernel-boundary timeline of one replay of the step's graph (nesf_trace_*): per kernel
    its stream and its end (and, after the first kernel of its stream, start) in ms."""
    import torch
    from nesf import api
    api.trace_enable(True)
    try:
        model.capture(precision)
        model.reset()
        model.graph_step()
        torch.cuda.synchronize()
        marks = api.trace_read()
    finally:
        api.trace_enable(False)
        model.capture(precision)
    r = lambda x: None if x is None else round(x, 3)
    return [{"kernel": n, "stream": s, "start_ms": r(b), "end_ms": r(e)} for n, s, b, e in api.timeline(marks)]


def kernel_time(model, precision, kernel, reps=10):
    """Mean duration (ms) of one kernel of the step, from trace events recorded on its stream
    around it in `reps` replays of the traced graph (its span runs from the previous mark on
    that stream)."""
    import torch
    from nesf import api
    api.trace_enable(True)
    spans = []
    try:
        model.capture(precision)
        for _ in range(reps):
            model.graph_step()
            torch.cuda.synchronize()
            for n, _, b, e in api.timeline(api.trace_read()):
                if n == kernel and b is not None:
                    spans.append(e - b)
    finally:
        api.trace_enable(False)
        model.capture(precision)
    return sum(spans) / len(spans) if spans else None


def error_stats(model, precision):
    """Max / p99 relative error of the fast solver against the plain FP64 solver on the full step
    outputs (normalised by max(|ref|, 1e-6 max|ref|)), over the cells where the plain solver
    converged: where it stops at maxiter its answer is its 100th iterate, which no other path
    reproduces (those cells are counted)."""
    import torch
    from nesf import fields as F
    L = model.layout
    res = {}
    model.reset()
    model.iterations = {k: torch.zeros(L.shape, dtype=torch.int32, device="cuda") for k in ("ao", "ai")}
    model.update_state("f64")
    torch.cuda.synchronize()
    its = {k: L.ring(v.cpu().numpy()) for k, v in model.iterations.items()}
    model.iterations = None
    conv = {"ao": its["ao"] < model.ao_spec.flux_formulation.solver_stop_criteria.maxiter,
            "ai": its["ai"] < model.ai_spec.flux_formulation.solver_stop_criteria.maxiter}
    res["nonconverged_cells_excluded"] = {k: int((~v).sum()) for k, v in conv.items()}
    ref = {("ao", k): L.ring(model.ao[k].double().cpu().numpy()) for k in F.AO_OUTPUTS}
    ref.update({("ai", k): L.ring(model.ai[k].double().cpu().numpy()) for k in F.AI_OUTPUTS})
    model.reset()
    model.update_state(precision)
    torch.cuda.synchronize()
    got = {("ao", k): L.ring(model.ao[k].double().cpu().numpy()) for k in F.AO_OUTPUTS}
    got.update({("ai", k): L.ring(model.ai[k].double().cpu().numpy()) for k in F.AI_OUTPUTS})
    for key, r in ref.items():
        g = got[key][conv[key[0]]]
        r = r[conv[key[0]]]
        den = np.maximum(np.abs(r), 1e-6 * np.abs(r).max())
        e = np.abs(g - r) / np.where(den > 0, den, 1.0)
        res[f"{key[0]}.{key[1]}"] = {"max": float(e.max()), "p99": float(np.percentile(e, 99))}
    model.reset()
    return res


HEADLINE_FLUXES = ("latent_heat", "sensible_heat", "water_vapor", "x_momentum", "y_momentum")


def step_snapshot(model, precision, row_index):
    """One coupling step from the initial state (the captured graph of `precision`), and the
    band rows `row_index` of every output it writes (interpolated atmosphere, the three
    interfaces, the net fluxes), as host FP64 arrays."""
    import torch
    from nesf.coupled import EXCHANGE_ATMOS
    model.capture(precision)
    model.reset()
    model.graph_step()
    torch.cuda.synchronize()
    grab = lambda t: t.index_select(0, row_index).double().cpu().numpy()
    snap = {"ao": {k: grab(v) for k, v in model.ao.items()}, "ai": {k: grab(v) for k, v in model.ai.items()},
            "io": {k: grab(v) for k, v in model.io.items()}, "net": {k: grab(v) for k, v in model.net.items()},
            "io_T": {"T_oc": grab(model.x["T_oc"])}}
    if model.atmos is not None:
        snap["atmos"] = {k: grab(model.x[k]) for k in EXCHANGE_ATMOS.values()}
    model.reset()
    return snap


def oracle_errors(model, precisions, bands=48, rows=8):
    """Max / p99 relative error of each precision's coupling step against the FP64 oracle
    (oracle/band.py: interpolation, the three interfaces, assembly and radiation restated on
    the CPU) on `bands` bands of `rows` rows spread over the workload, per output. Relative
    error = |gpu - oracle| / max(|oracle|, 1e-6 max|oracle|); interface temperatures in kelvin.

    Three tables per precision:
      solver       the oracle solves from the atmosphere the GPU interpolated (the FP32
                   values the GPU's solves read): the solvers' and the assembly's error on
                   the same inputs -- the accuracy the metric states;
      interpolation the GPU's FP32 interpolation (FP32 arithmetic, as the reference's Float32
                   kernels) against the oracle's FP64 one;
      end_to_end   everything from the oracle's own FP64 interpolation: the solves then
                   amplify the interpolated inputs' FP32 rounding where differences cancel.
    Cells where the oracle's atmosphere-ocean or atmosphere-sea-ice iteration stops at maxiter
    are excluded and counted: there the reference's answer is its 100th iterate, which the
    warm-started path need not follow. The net momentum fluxes also read the west / south
    neighbours' interface stress, so they exclude the neighbours of such cells too."""
    import torch
    from oracle import band as OB
    st = model.state
    L = model.layout
    h = rows + 2 * L.hy
    pos = OB.band_positions(st, rows, bands)
    row_index = torch.cat([torch.arange(int(p), int(p) + h) for p in pos]).cuda()
    snaps = {p: step_snapshot(model, p, row_index) for p in precisions}
    tables = {p: {t: OB.ErrorTable() for t in ("solver", "interpolation", "end_to_end")} for p in precisions}
    maxit = {"ao": model.ao_spec.flux_formulation.solver_stop_criteria.maxiter,
             "ai": model.ai_spec.flux_formulation.solver_stop_criteria.maxiter}
    kelvin = lambda k, a: a + 273.15 if k == "interface_temperature" else a
    specs = (model.ao_spec, model.ai_spec, model.io_spec, model.asm_spec)
    excluded = 0
    t0 = time.perf_counter()
    for b, lo in enumerate(pos):
        part = lambda a: a[b * h:(b + 1) * h]
        _, own = OB.step_band(st, int(lo), rows, *specs)
        for p, snap in snaps.items():
            sub, same = OB.step_band(st, int(lo), rows, *specs,
                                     atmos={k: part(v) for k, v in snap.get("atmos", {}).items()})
            I = sub.interior
            for table, ref in (("solver", same), ("end_to_end", own)):
                stopped = (I(ref["ao"]["iterations"]) >= maxit["ao"]) | (I(ref["ai"]["iterations"]) >= maxit["ai"])
                if table == "solver" and p == precisions[0]:
                    excluded += int(stopped.sum())
                near = stopped.copy()
                near[:, 1:] |= stopped[:, :-1]
                near[1:, :] |= stopped[:-1, :]
                for group in ("ao", "ai", "io", "net"):
                    if group not in ref or group not in snap:
                        continue
                    for k, r in ref[group].items():
                        if k == "iterations" or k not in snap[group]:
                            continue
                        tables[p][table].add(f"{group}.{k}", kelvin(k, I(part(snap[group][k]))), kelvin(k, I(r)),
                                             ~near if group == "net" else ~stopped)
                tables[p][table].add("io.ocean_T_after_frazil", I(part(snap["io_T"]["T_oc"])),
                                     I(ref["io"]["T_oc"][0]), ~stopped)
            for k, r in own.get("atmos", {}).items():
                tables[p]["interpolation"].add(f"atmos.{k}", I(part(snap["atmos"][k])), I(r))
    oracle_s = time.perf_counter() - t0
    out = {}
    for p, t in tables.items():
        s = {name: tab.summary() for name, tab in t.items()}
        head = [s["solver"][f"{g}.{k}"] for g in ("ao", "ai") for k in HEADLINE_FLUXES if f"{g}.{k}" in s["solver"]]
        out[p] = {"max_headline_fluxes": max(x["max"] for x in head),
                  "p99_headline_fluxes": max(x["p99"] for x in head), **s}
    out["sample"] = (f"{len(pos)} bands of {rows} rows x {L.nx} cells spread over the domain; "
                     f"{excluded} cells where the oracle stops at maxiter excluded; oracle {oracle_s:.1f} s "
                     f"on {_oracle_threads()} threads")
    return out


# ------------------------------------------------------------ the other configurations
CONFIG_WORKLOADS = {
    0: "ao_1deg: 360x180 (1 degree) atmosphere-ocean, no land, atmosphere on the exchange grid, FP64 fields",
    1: "ao_quarter_land: 1440x560 (lat -70..70) atmosphere-ocean, 30% land, 640x320x2 prescribed atmosphere "
       "interpolated onto the grid, FP32 fields",
    2: "coupled_1440: 1440x600 (lat -75..75) atmosphere-ocean + atmosphere-sea-ice + sea-ice-ocean fluxes and "
       "the net-flux assembly with radiation in one coupling step (CUDA graph), FP32 fields",
    3: "ensemble_32: 32 members x 720x360 atmosphere-ocean in one launch, each member with its own Charnock "
       "parameter, gustiness and roughness coefficients, per-member FP64 compensated integrals, FP32 fields",
}


class AOStep:
    """An atmosphere-ocean step (with the interpolation of a prescribed atmosphere when the
    workload has one) on the device, captured as one coupling-step graph."""

    def __init__(self, state):
        import torch
        from nesf import api
        from nesf import fields as F
        from nesf import params as P
        from nesf.coupled import ATMOS_NAMES, EXCHANGE_ATMOS
        self.state, self.layout = state, state.layout
        self.spec = P.atmosphere_ocean_interface_spec()
        self.x = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in state.fields.items()}
        dt = self.x["u_oc"].dtype
        interp = None
        if state.atmos is not None:
            self.src = {n: torch.from_numpy(state.atmos["arrays"][n]).cuda() for n in ATMOS_NAMES}
            for n in ATMOS_NAMES:
                self.x[EXCHANGE_ATMOS[n]] = torch.zeros(self.layout.shape, dtype=dt, device="cuda")
            interp = (state.coords, state.atmos, self.src, {n: self.x[EXCHANGE_ATMOS[n]] for n in ATMOS_NAMES},
                      None, state.atmos["time_weight"])
        self.ao = {k: torch.zeros(self.layout.shape, dtype=dt, device="cuda") for k in F.AO_OUTPUTS}
        arrays = {k: self.x.get(k) for k in F.AO_INPUTS}
        arrays.update(self.ao)
        self.step = api.CouplingStep(self.spec, self.layout, arrays, interp=interp)
        self.graphs = {}

    def cells(self):
        return int((self.layout.interior(self.state.fields["inactive"]) == 0).sum())

    def graph(self, precision):
        from nesf import api
        if precision not in self.graphs:
            self.graphs[precision] = api.Graph(self.step, precision)
        return self.graphs[precision]


def time_graph(launch, steps, warmup):
    """ms per launch of `launch()`, CUDA events on the current stream after `warmup` launches."""
    import torch
    for _ in range(warmup):
        launch()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        launch()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _ao_band_errors(table, got, state, lo, rows, ref, keep):
    from oracle import band as OB
    sub, rs = OB.band_rows(state, lo, rows)
    kelvin = lambda k, a: a + 273.15 if k == "interface_temperature" else a
    for k in HEADLINE_FLUXES + ("friction_velocity", "temperature_scale", "water_vapor_scale",
                                "interface_temperature"):
        table.add(f"ao.{k}", kelvin(k, sub.interior(np.asarray(got[k])[rs])), kelvin(k, sub.interior(ref[k])), keep)


def _summary(table):
    s = table.summary()
    head = [v for k, v in s.items() if k.split(".")[1] in HEADLINE_FLUXES]
    return {"max_headline_fluxes": max(v["max"] for v in head), "p99_headline_fluxes": max(v["p99"] for v in head),
            "per_output": s}


def config_entry(n, steps=20):
    """Throughput, accuracy against the oracle and the oracle's CPU rate for configuration n
    (0-3), whose workload CONFIG_WORKLOADS names: the adaptive FP32 solver (no warm start) and
    the plain FP64 solver on the GPU, the oracle on bands of rows on the host cores."""
    import torch
    from nesf import api
    from nesf import fields as F
    from nesf import params as P
    from nesf import synthetic as syn
    from nesf.coupled import CoupledModel, EXCHANGE_ATMOS
    from oracle import band as OB
    from oracle import oracle
    rows = 8
    out = {"workload": CONFIG_WORKLOADS[n]}
    if n == 3:
        st = syn.ensemble()
        L = st.layout
        specs = [syn.ensemble_member_spec(p) for p in st.perturbations]
        dev = api.to_device({k: st.fields[k] for k in F.AO_INPUTS if k in st.fields})
        res = {k: torch.zeros((st.members,) + L.shape, dtype=torch.float32, device="cuda") for k in F.AO_OUTPUTS}
        cells = int((np.stack([L.interior(m) for m in st.fields["inactive"]]) == 0).sum())
        run = lambda prec: (lambda: api.compute_atmosphere_ocean_fluxes_ensemble(specs, L, dev, res, precision=prec))
        ms = {p: time_graph(run(p), steps if p != "f64" else max(3, steps // 4), 2) for p in ("f32_adaptive", "f64")}
        lat = st.coords.lat0 + np.arange(L.ny) * st.coords.dlat
        rows_dev = torch.from_numpy(np.cos(np.radians(lat)) * 1.0e10).cuda()
        tables = {}
        for prec in ("f32_adaptive", "f64"):
            run(prec)()
            torch.cuda.synchronize()
            got = {k: v.double().cpu().numpy() for k, v in res.items()}
            t = OB.ErrorTable()
            cpu_s, cpu_cells = 0.0, 0
            for mbr in range(st.members):
                ms_state = syn.SurfaceState(L, st.coords, st.dtype, fields={k: v[mbr] for k, v in st.fields.items()})
                lo = int(OB.band_positions(ms_state, rows, st.members)[mbr])
                t0 = time.perf_counter()
                sub, ref = OB.step_band(ms_state, lo, rows, specs[mbr])
                cpu_s += time.perf_counter() - t0
                cpu_cells += int((sub.interior(ref["inputs"]["inactive"]) == 0).sum())
                keep = sub.interior(ref["ao"]["iterations"]) < 100
                _ao_band_errors(t, {k: v[mbr] for k, v in got.items()}, ms_state, lo, rows, ref["ao"], keep)
            tables[prec] = _summary(t)
        integrals = []
        for mbr in range(st.members):
            r = api.area_integrals(L, [res["sensible_heat"][mbr], res["latent_heat"][mbr]],
                                   row_area=rows_dev).cpu().numpy()
            integrals.append([float(r[0][0]), float(r[1][0])])
        out.update(cells=cells, members=st.members, integrals_sensible_latent=integrals[:4],
                   integrals_note="per-member compensated FP64 sums (sum, residual pairs on the device) of the "
                                  "last solve's sensible and latent heat, rows weighted by cos(lat); first 4 shown")
    elif n in (0, 1):
        st = syn.ao_1deg() if n == 0 else syn.ao_quarter_land()
        m = AOStep(st)
        cells = m.cells()
        ms = {p: time_graph(m.graph(p).launch, steps if p != "f64" else max(3, steps // 4), 3)
              for p in ("f32_adaptive", "f64")}
        tables = {}
        cpu_s, cpu_cells = 0.0, 0
        for prec in ("f32_adaptive", "f64"):
            m.graph(prec).launch()
            torch.cuda.synchronize()
            got = {k: v.double().cpu().numpy() for k, v in m.ao.items()}
            atm = {k: m.x[k].double().cpu().numpy() for k in EXCHANGE_ATMOS.values()} if st.atmos is not None else None
            t = OB.ErrorTable()
            for lo in OB.band_positions(st, rows, 16):
                _, rs = OB.band_rows(st, int(lo), rows)
                t0 = time.perf_counter()
                sub, ref = OB.step_band(st, int(lo), rows, m.spec,
                                        atmos=None if atm is None else {k: v[rs] for k, v in atm.items()})
                if prec == "f64":
                    cpu_s += time.perf_counter() - t0
                    cpu_cells += int((sub.interior(ref["inputs"]["inactive"]) == 0).sum())
                keep = sub.interior(ref["ao"]["iterations"]) < 100
                _ao_band_errors(t, got, st, int(lo), rows, ref["ao"], keep)
            tables[prec] = _summary(t)
    else:
        st = syn.coupled_1440()
        m = CoupledModel(st)
        n_ao, n_ai = m.active_cells()
        cells = n_ao + n_ai
        ms = {}
        for p in ("f32_adaptive", "f64"):
            m.capture(p)
            ms[p] = time_graph(m.graph_step, steps if p != "f64" else max(3, steps // 4), 3)
        ev = oracle_errors(m, ["f32_adaptive", "f64"], bands=16, rows=rows)
        tables = {p: {"max_headline_fluxes": ev[p]["max_headline_fluxes"],
                      "p99_headline_fluxes": ev[p]["p99_headline_fluxes"],
                      "per_output": ev[p]["solver"]} for p in ("f32_adaptive", "f64")}
        t0 = time.perf_counter()
        cpu_cells = 0
        sp = (m.ao_spec, m.ai_spec, m.io_spec, m.asm_spec)
        for lo in OB.band_positions(st, rows, 16):
            sub, ref = OB.step_band(st, int(lo), rows, *sp)
            water = sub.interior(ref["inputs"]["inactive"]) == 0
            ice = sub.interior(ref["inputs"]["ice_concentration"]) > 0
            cpu_cells += int(water.sum() + (water & ice).sum())
        cpu_s = time.perf_counter() - t0
    out.update(cells=cells, fast_ms_per_step=ms["f32_adaptive"], plain_f64_ms_per_step=ms["f64"],
               fast_cells_per_s=cells / (ms["f32_adaptive"] / 1000.0), plain_f64_cells_per_s=cells / (ms["f64"] / 1000.0),
               speedup_vs_plain_f64=ms["f64"] / ms["f32_adaptive"],
               errors_vs_oracle={"fast": tables["f32_adaptive"], "plain_f64": tables["f64"]},
               cpu_oracle={"cells_per_s": cpu_cells / cpu_s if cpu_s > 0 else None, "cores": oracle.get_threads(),
                           "sample": f"{cpu_cells} solved cells on bands of {rows} rows, {cpu_s:.2f} s"})
    torch.cuda.synchronize()
    return out


def _oracle_threads():
    from oracle import oracle
    return oracle.get_threads()


def e2e_step_time(model, precision, steps, warmup):
    """Same step through the public API with host buffers: pinned H2D of the step's inputs
    (ocean and sea-ice surface state + the two atmosphere snapshots) into the model's
    fields, the captured step (nesf_graph_launch), and a D2H read of the net boundary
    fluxes, all inside the timed region."""
    import torch
    from nesf.coupled import ICE_NET, OCEAN_NET, STEP_INPUTS
    names = [k for k in STEP_INPUTS if k in model.x]
    host_in = {k: model.x[k].cpu().pin_memory() for k in names}
    atm_in = {k: v.cpu().pin_memory() for k, v in model.atmos_src.items()} if model.atmos is not None else {}
    host_out = {k: torch.empty_like(model.net[k], device="cpu").pin_memory() for k in OCEAN_NET + ICE_NET}
    h2d = sum(t.numel() * t.element_size() for t in host_in.values()) + \
        sum(t.numel() * t.element_size() for t in atm_in.values())
    d2h = sum(t.numel() * t.element_size() for t in host_out.values())
    s = torch.cuda.current_stream()

    model.capture(precision)

    def one():
        for k, t in host_in.items():
            model.x[k].copy_(t, non_blocking=True)
        for k, t in atm_in.items():
            model.atmos_src[k].copy_(t, non_blocking=True)
        model.graph_step()
        for k, t in host_out.items():
            t.copy_(model.net[k], non_blocking=True)

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        one()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, h2d, d2h


def e2e_pipelined_step_time(models, precision, steps, warmup):
    """The same end-to-end step, double-buffered: two models (two sets of fields and two
    captured graphs) alternate; while one slot's graph runs on the compute stream, a copy
    stream moves the next step's inputs into the other slot (pinned H2D) and the previous
    step's net fluxes out (D2H). Every step still copies all its inputs in and its result
    out inside the timed region, which runs from the first copy to the last."""
    import torch
    from nesf.coupled import ICE_NET, OCEAN_NET, STEP_INPUTS
    a = models[0]
    names = [k for k in STEP_INPUTS if k in a.x]
    host_in = {k: a.x[k].cpu().pin_memory() for k in names}
    atm_in = {k: v.cpu().pin_memory() for k, v in a.atmos_src.items()} if a.atmos is not None else {}
    host_out = [{k: torch.empty_like(a.net[k], device="cpu").pin_memory() for k in OCEAN_NET + ICE_NET}
                for _ in models]
    h2d = sum(t.numel() * t.element_size() for t in host_in.values()) + \
        sum(t.numel() * t.element_size() for t in atm_in.values())
    d2h = sum(t.numel() * t.element_size() for t in host_out[0].values())
    # inputs and results on separate copy streams, so that the next step's H2D does not
    # queue behind the D2H of the step still computing
    comp, copy, back = torch.cuda.current_stream(), torch.cuda.Stream(), torch.cuda.Stream()
    for m in models:
        m.capture(precision)
    ev_in = [torch.cuda.Event() for _ in models]
    ev_done = [torch.cuda.Event() for _ in models]
    ev_out = [torch.cuda.Event() for _ in models]
    for e in ev_done + ev_out:
        e.record(comp)

    def run(n_steps):
        for n in range(n_steps):
            i = n % 2
            m = models[i]
            with torch.cuda.stream(copy):
                copy.wait_event(ev_done[i])            # the slot's previous graph has read its inputs
                for k, t in host_in.items():
                    m.x[k].copy_(t, non_blocking=True)
                for k, t in atm_in.items():
                    m.atmos_src[k].copy_(t, non_blocking=True)
                ev_in[i].record(copy)
            comp.wait_event(ev_in[i])
            comp.wait_event(ev_out[i])                 # the slot's previous result has been read out
            m.graph_step(stream=comp)
            ev_done[i].record(comp)
            with torch.cuda.stream(back):
                back.wait_event(ev_done[i])
                for k, t in host_out[i].items():
                    t.copy_(m.net[k], non_blocking=True)
                ev_out[i].record(back)
        comp.wait_stream(copy)
        comp.wait_stream(back)

    run(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    copy.wait_event(e0)
    back.wait_event(e0)
    run(steps)
    e1.record(comp)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, h2d, d2h


def cpu_baseline(state, target_s=12.0):
    """The oracle (C restatement, OpenMP over all host threads) on bands of rows of the same
    workload, every phase of the GPU step (oracle/band.py): interpolation of the prescribed
    atmosphere onto the band, the atmosphere-ocean, atmosphere-sea-ice and sea-ice-ocean
    fluxes, the net ocean and sea-ice assembly with radiation; returns solved cells/s (the
    GPU step's unit) and the sample."""
    from nesf import params as P
    from oracle import band as OB
    from oracle import oracle
    L = state.layout
    f = state.fields
    rows = 8
    threads = oracle.get_threads()
    done_cells = 0
    elapsed = 0.0
    hist = {}
    specs = dict(ao_spec=P.atmosphere_ocean_interface_spec(), ai_spec=P.atmosphere_sea_ice_interface_spec(),
                 io_spec=P.SeaIceOceanSpec(), asm_spec=P.AssemblySpec())
    positions = OB.band_positions(state, rows, 97)
    bands = 0
    while elapsed < target_s and bands < 10 * len(positions):
        lo = int(positions[bands % len(positions)])
        t0 = time.perf_counter()
        sub, res = OB.step_band(state, lo, rows, **specs)
        elapsed += time.perf_counter() - t0
        water = sub.interior(OB.band_of(f["inactive"], state, lo, rows)) == 0
        ice = sub.interior(OB.band_of(f["ice_concentration"], state, lo, rows)) > 0
        done_cells += int(water.sum() + (water & ice).sum())
        for name, sel in (("ao", water), ("ai", water & ice)):
            h = hist.setdefault(name, np.zeros(len(ITER_BINS) - 1, dtype=np.int64))
            h += np.histogram(sub.interior(res[name]["iterations"])[sel], bins=ITER_BINS)[0]
        bands += 1
    return {"value": done_cells / elapsed, "unit": "flux cells/s", "cores": threads, "kind": "port",
            "nproc": os.cpu_count(), "cpu_model": cpu_model(),
            "iteration_histogram": {"bins": ITER_BINS.tolist(), **{k: v.tolist() for k, v in hist.items()}},
            "sample": f"{bands} bands of {rows} rows x {L.nx} cells spread over the domain ({done_cells} "
                      f"solved cells): the whole step (interpolation, AO + AI + IO fluxes, assembly and "
                      f"radiation), {elapsed:.1f} s of CPU work"}


ITER_BINS = np.array([1, 3, 5, 8, 12, 16, 20, 30, 50, 100, 101])


def cpu_model():
    """The host CPU's model name (/proc/cpuinfo; on Arm the implementer and part numbers)."""
    try:
        with open("/proc/cpuinfo") as fh:
            info = fh.read()
    except OSError:
        return "unknown"
    for key in ("model name", "Model"):
        for line in info.splitlines():
            if line.startswith(key) and ":" in line:
                return line.split(":", 1)[1].strip()
    parts = {}
    for line in info.splitlines():
        if ":" in line:
            k, v = (x.strip() for x in line.split(":", 1))
            if k in ("CPU implementer", "CPU part") and k not in parts:
                parts[k] = v
    return ", ".join(f"{k} {v}" for k, v in parts.items()) or "unknown"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    state = make_state(args.small)
    for _ in range(args.warmup):
        cpu_baseline(state, target_s=0.5)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(state, target_s=max(1.0, 60.0 / max(1, args.steps))))
    wall = time.perf_counter() - t0
    v = float(np.mean([x["value"] for x in vals]))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "flux cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": "row bands of the workload", "parallelism": "openmp"},
            "cpu_baseline": {"value": v, "unit": "flux cells/s", "cores": oracle.get_threads(), "kind": "port",
                             "nproc": vals[-1]["nproc"], "cpu_model": vals[-1]["cpu_model"],
                             "iteration_histogram": vals[-1]["iteration_histogram"],
                             "sample": vals[-1]["sample"] + " (the reference is Julia; no Julia toolchain here)"},
            "e2e": {"value": v, "unit": "flux cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    from nesf.coupled import CoupledModel
    state = make_state(args.small)
    model = CoupledModel(state)
    n_ao, n_ai = model.active_cells()
    cells = n_ao + n_ai
    prec = args.precision
    warm_info = None
    if prec != "f64" and not args.cold:
        model.mlp, warm_info = train_warm_start(samples=args.warm_samples)
    # launch shapes and schedule from the autotuner (nesf_autotune), on this workload
    tuning = model.autotune(prec, reps=3) if not args.no_autotune else None

    # warm-up, then the timed region (fast path: exactly `steps` replays, the headline), then
    # REPEAT_ROUNDS - 1 more rounds of `steps` replays for the spread; clocks sampled throughout
    with ClockSampler(local) as clocks:
        ms, launches = time_steps(model, prec, args.steps, args.warmup, world)
        rounds = [ms] + [replay_round(model, args.steps, world) for _ in range(REPEAT_ROUNDS - 1)]
    clk = clocks.summary()
    if args.no_plain:
        print(json.dumps({"metric": METRIC, "value": cells * world / (ms / 1000.0), "unit": "flux cells/s",
                          "ms_per_step": ms, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "note": "profiling run: --precision only"}))
        return
    mlp, model.mlp = model.mlp, None          # the comparison arms run from the cold start
    ms_plain, _ = time_steps(model, "f64", max(3, args.steps // 4), 3, world)
    ms_polish = time_steps(model, "f32", max(3, args.steps // 4), 3, world)[0]
    ms_cold = time_steps(model, prec, max(3, args.steps // 4), 3, world)[0] if mlp is not None else ms
    model.mlp = mlp
    phases = phase_times(model, prec)
    phases_plain = phase_times(model, "f64", reps=1)
    value = cells * world / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": "flux cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"f32": "f32+f64polish", "f32_adaptive": "f32 (f64 polish where ill-conditioned)"}.get(prec, "f64"), "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells_ao": n_ao, "cells_ai": n_ai, "fields": "fp32",
                       "warm_start": model.mlp is not None,
                       "schedule": "one thread per cell (sea-ice pass 1: resident warps taking 32 work-list "
                                   "entries at a time), compacted work lists, packed polish/replay passes; "
                                   "sea-ice and ocean solves on two lanes (the ocean solve overlaps the sea-ice "
                                   "polish/replay tail); the step replayed as one CUDA graph",
                       "l2": "working set > L2 (no flush needed)", "parallelism": f"replicas x{world}",
                       "tuning": tuning},
            "gpu_launches": launches,
            "clocks": clk,
            "repeat_rounds": {"rounds": len(rounds), "steps_per_round": args.steps,
                              "ms_per_step": [round(x, 4) for x in rounds], "median": float(np.median(rounds)),
                              "min": min(rounds), "max": max(rounds),
                              "note": "the headline ms_per_step is the first round"},
            "plain_f64": {"value": cells * world / (ms_plain / 1000.0), "ms_per_step": ms_plain,
                          "phases_ms": phases_plain},
            "f32_polish_ms_per_step": ms_polish,
            "cold_start_ms_per_step": ms_cold,
            "warm_start": warm_info,
            "phases_ms": phases}
    if rank == 0:
        line["speedup_vs_plain_f64"] = ms_plain / ms
        line["timeline"] = step_timeline(model, prec)
        model.reset()
        s_ao, s_ai = model.compute_fluxes(prec, stats=True)
        model.reset()
        mlp, model.mlp = model.mlp, None
        c_ao, c_ai = model.compute_fluxes(prec, stats=True)
        model.reset()
        p_ao, p_ai = model.compute_fluxes("f64", stats=True)
        model.mlp = mlp
        model.reset()
        strip = lambda d: {k: (v if not hasattr(v, "tolist") else v.tolist()) for k, v in d.items() if k != "histogram"}
        line["solver_stats"] = {"ao": strip(s_ao), "ai": strip(s_ai), "ao_cold": strip(c_ao), "ai_cold": strip(c_ai),
                                "ao_plain": strip(p_ao), "ai_plain": strip(p_ai)}
        per = lambda d: d["iterations"] / max(1, d["solved"])
        line["iterations_per_cell"] = {"ao": per(s_ao), "ao_cold": per(c_ao), "ai": per(s_ai), "ai_cold": per(c_ai),
                                       "ao_plain": per(p_ao), "ai_plain": per(p_ai)}
        line["errors_vs_plain_f64"] = error_stats(model, prec)
        ev = oracle_errors(model, [prec, "f64"])
        line["errors_vs_oracle"] = {"fast": ev[prec], "plain_f64": ev["f64"], "sample": ev["sample"]}
        line["max_rel_err_vs_oracle"] = ev[prec]["max_headline_fluxes"]
        # roofline of the main solve kernel, the atmosphere-ocean pass 1 (ao_adaptive_kernel), timed with
        # trace events on its stream inside graph replays. It is bound by the latency of its
        # FP32 arithmetic, not by HBM: the HBM fraction is small, and the
        # work-table rate (transcendentals and flops per second, NESF_WORK_*) is given beside it.
        from nesf import _abi as A
        peaks, kind = measured_peaks()
        t_ao = kernel_time(model, prec, "ao_pass1")
        W = A.WORK
        alg = W["BYTES_PER_CELL_F32"] * n_ao
        it_ao = p_ao["iterations"]   # FP64 cold-start iterations of the solved cells
        work_t = n_ao * (W["PROLOGUE_TRANSCENDENTALS"] + W["EPILOGUE_TRANSCENDENTALS"]) + it_ao * W["ITER_TRANSCENDENTALS"]
        work_f = n_ao * (W["PROLOGUE_FLOPS"] + W["EPILOGUE_FLOPS"]) + it_ao * W["ITER_FLOPS"]
        achieved = alg / (t_ao / 1000.0) / 1e9 if t_ao else None
        traffic = AO_KERNEL_DRAM_BYTES_PER_CELL * n_ao if AO_KERNEL_DRAM_BYTES_PER_CELL else None
        line["roofline"] = {"bound": "hbm", "kernel": "ao_adaptive_kernel<float, bulk> (atmosphere-ocean pass 1)",
                            "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                            "frac": achieved / peaks["hbm_gbs"] if achieved else None, "traffic": traffic,
                            "algorithmic_bytes": alg, "kernel_ms": t_ao, "peak_source": kind,
                            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                                              "on the 720x320 case, scaled by cells; above the algorithmic "
                                              "bytes: the classify pass's 64-byte record per cell",
                            "compute": compute_roofline(work_t, work_f, t_ao, it_ao, clk)}
        if not args.no_e2e:
            ms_ser, h2d, d2h = e2e_step_time(model, prec, max(3, args.steps // 2), 1)
            twin = CoupledModel(state)                 # the second slot of the double buffer
            twin.mlp = model.mlp
            ms_e2e, h2d, d2h = e2e_pipelined_step_time([model, twin], prec, max(10, args.steps), 2)
            del twin
            line["e2e"] = {"value": cells / (ms_e2e / 1000.0), "unit": "flux cells/s", "h2d_bytes_per_step": h2d,
                           "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e,
                           "mode": "double-buffered: step n+1's H2D and step n-1's D2H on two copy streams "
                                   "beside step n's graph",
                           "serial_ms_per_step": ms_ser}
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(state)
        if not args.no_configs:
            # the other configurations of the same metric, beside this one (configuration 4)
            line["configs"] = {str(n): config_entry(n) for n in (0, 1, 2, 3)}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
