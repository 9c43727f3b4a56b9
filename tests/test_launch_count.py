"""The number of kernels a coupling step launches (`CoupledModel.kernels_per_step`, the
bench's `gpu_launches` per step), against the kernel lists of the step written out by
hand from the library's launch order:

* native adaptive step with the warm start (the bench's workload), 16 kernels:
  interpolation; sea ice: classify, pass 1, polish, pass 1's replays, the polish pass's
  replays; ocean: classify, warm-start inference, pass 1, polish, the two replay passes;
  sea-ice-ocean fluxes and the frazil adjustment; ocean and sea-ice assembly, each with
  its radiative add-on inside;
* the same step through the per-phase entry points: one sea-ice-ocean kernel, and the
  two radiative add-ons as kernels of their own (17);
* plain FP64: classify and solve per interface (9 native, 10 per phase).
Host logic only: no GPU, no library."""
from nesf.coupled import CoupledModel


def model(mlp=True, atmos=True):
    m = CoupledModel.__new__(CoupledModel)   # the launch count reads only these two
    m.mlp = object() if mlp else None
    m.atmos = object() if atmos else None
    return m


NATIVE_ADAPTIVE_WARM = ["interp_tile",
                        "ai_classify", "ai_adaptive", "ai_polish", "ai_replay (pass 1)", "ai_replay (polish)",
                        "ao_classify", "mlp_infer", "ao_adaptive", "ao_polish", "ao_replay (pass 1)",
                        "ao_replay (polish)",
                        "io_fluxes", "io_frazil",
                        "assemble_ocean (+ radiation)", "assemble_ice (+ radiation)"]


def test_native_adaptive_step_with_warm_start():
    assert model().kernels_per_step("f32_adaptive", native=True) == len(NATIVE_ADAPTIVE_WARM) == 16


def test_per_phase_adaptive_step():
    # one sea-ice-ocean kernel (fluxes and frazil together), the radiative add-ons apart
    n = len(NATIVE_ADAPTIVE_WARM) - 1 + 2
    assert model().kernels_per_step("f32_adaptive") == n == 17


def test_cold_start_and_plain():
    assert model(mlp=False).kernels_per_step("f32_adaptive", native=True) == 15
    assert model().kernels_per_step("f64", native=True) == 1 + 2 * 2 + 2 + 2
    assert model().kernels_per_step("f64") == 1 + 2 * 2 + 1 + 4
    assert model(atmos=False).kernels_per_step("f64", native=True) == 2 * 2 + 2 + 2
