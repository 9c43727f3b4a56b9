"""The autotuner (nesf_autotune) and the tunings it chooses between: every launch
shape and schedule gives bit-identical outputs (the cells' arithmetic does not
depend on them), and the search sets a valid, timed tuning on the context."""
import numpy as np
import pytest

from helpers import to_numpy
from nesf import api
from nesf import fields as F
from nesf import synthetic as syn
from nesf.coupled import CoupledModel, ICE_NET, OCEAN_NET, RAD_DIAG

pytestmark = pytest.mark.gpu

DEFAULT = dict(solve_block=128, deferred_per_sm=4, infer_per_sm=4, two_lanes=1, io_overlap=1, pass1_fetch=2,
               refill_lanes=8, early_ocean_classify=0, ice_deferred_per_sm=0, cells_per_thread=1)


@pytest.fixture(scope="module")
def model():
    st = syn.coupled(seed=43, nx=240, ny=120, lat_s=-80, lat_n=80, land=0.3, interpolate=True)
    m = CoupledModel(st)
    yield m
    api.set_tuning(**DEFAULT)


def outputs(m):
    import torch
    torch.cuda.synchronize()
    out = {("ao", k): to_numpy(m.ao[k]).copy() for k in F.AO_OUTPUTS}
    out.update({("ai", k): to_numpy(m.ai[k]).copy() for k in F.AI_OUTPUTS})
    out[("ai", "interface_temperature")] = to_numpy(m.ai["interface_temperature"]).copy()
    out.update({("io", k): to_numpy(m.io[k]).copy() for k in F.IO_OUTPUTS})
    out.update({("net", k): to_numpy(m.net[k]).copy() for k in OCEAN_NET + ICE_NET + RAD_DIAG})
    out[("x", "T_oc")] = to_numpy(m.x["T_oc"]).copy()
    return out


def step(m, precision, **tuning):
    api.set_tuning(**{**DEFAULT, **tuning})
    m.reset()
    m.native_step(precision)
    return outputs(m)


@pytest.mark.parametrize("precision", ["f64", "f32", "f32_adaptive"])
def test_every_tuning_gives_the_same_outputs(model, precision):
    ref = step(model, precision)
    for tuning in (dict(solve_block=32), dict(solve_block=64, deferred_per_sm=16), dict(deferred_per_sm=1),
                   dict(two_lanes=0), dict(io_overlap=0), dict(two_lanes=0, io_overlap=0, solve_block=96),
                   dict(pass1_fetch=1), dict(pass1_fetch=3), dict(pass1_fetch=3, solve_block=64),
                   dict(pass1_fetch=2, solve_block=32), dict(pass1_fetch=4), dict(pass1_fetch=4, refill_lanes=1),
                   dict(pass1_fetch=4, refill_lanes=16, solve_block=64), dict(pass1_fetch=4, refill_lanes=3),
                   dict(early_ocean_classify=1), dict(early_ocean_classify=1, two_lanes=0),
                   dict(early_ocean_classify=2), dict(early_ocean_classify=2, io_overlap=0),
                   dict(early_ocean_classify=3), dict(early_ocean_classify=3, io_overlap=0),
                   dict(ice_deferred_per_sm=1), dict(ice_deferred_per_sm=2, deferred_per_sm=8),
                   dict(cells_per_thread=2), dict(cells_per_thread=4, pass1_fetch=1),
                   dict(cells_per_thread=3, pass1_fetch=3, solve_block=64),
                   dict(cells_per_thread=8, pass1_fetch=4, refill_lanes=5)):
        got = step(model, precision, **tuning)
        for k in ref:
            assert np.array_equal(ref[k], got[k], equal_nan=True), (precision, tuning, k)


def test_warm_start_inference_grid(model):
    from nesf.warm import WarmStartNetwork
    model.mlp = WarmStartNetwork(seed=3)
    try:
        ref = step(model, "f32_adaptive")
        for tuning in (dict(infer_per_sm=1), dict(infer_per_sm=2), dict(infer_per_sm=8), dict(pass1_fetch=4),
                       dict(pass1_fetch=4, refill_lanes=5), dict(early_ocean_classify=1), dict(early_ocean_classify=2),
                       dict(early_ocean_classify=3),
                       dict(cells_per_thread=2, pass1_fetch=3), dict(cells_per_thread=4, pass1_fetch=1)):
            got = step(model, "f32_adaptive", **tuning)
            for k in ref:
                assert np.array_equal(ref[k], got[k], equal_nan=True), (tuning, k)
    finally:
        model.mlp = None


def test_autotune_sets_a_valid_tuning(model):
    api.set_tuning(**DEFAULT)
    model.reset()
    model.native_step("f32_adaptive")
    ref = outputs(model)
    t = model.autotune("f32_adaptive", reps=2)
    assert t["step_ms"] > 0
    assert t["solve_block"] in (32, 64, 96, 128) and 1 <= t["deferred_per_sm"] <= 16
    assert t["two_lanes"] in (0, 1) and t["io_overlap"] in (0, 1) and t["pass1_fetch"] in (1, 2, 3, 4)
    assert 1 <= t["refill_lanes"] <= 32 and t["early_ocean_classify"] in (0, 1, 2, 3)
    assert 0 <= t["ice_deferred_per_sm"] <= 16 and 1 <= t["cells_per_thread"] <= 8
    cur = api.get_tuning()
    assert {k: cur[k] for k in DEFAULT} == {k: t[k] for k in DEFAULT}
    model.reset()
    model.native_step("f32_adaptive")
    got = outputs(model)
    for k in ref:
        assert np.array_equal(ref[k], got[k], equal_nan=True), k


def test_graph_keeps_its_tuning(model):
    """A graph captured under one tuning replays it after the context's tuning changes."""
    ref = step(model, "f32_adaptive", two_lanes=0)
    model.capture("f32_adaptive")
    api.set_tuning(**DEFAULT)
    model.reset()
    model.graph_step()
    got = outputs(model)
    for k in ref:
        assert np.array_equal(ref[k], got[k], equal_nan=True), k


def test_autotune_through_the_cache(model, tmp_path):
    """The first cached autotune searches and records; the second sets the recorded tuning
    without a step; the key names this device and step."""
    import torch
    path = tmp_path / "tuning.bin"
    api.set_tuning(**DEFAULT)
    first = model.autotune("f32_adaptive", reps=1, cache=path)
    assert first["from_cache"] is False and first["step_ms"] > 0
    api.set_tuning(**dict(DEFAULT, solve_block=32, two_lanes=0))
    second = model.autotune("f32_adaptive", reps=1, cache=path)
    assert second["from_cache"] is True
    assert {k: second[k] for k in DEFAULT} == {k: first[k] for k in DEFAULT}
    cur = api.get_tuning()
    assert {k: cur[k] for k in DEFAULT} == {k: first[k] for k in DEFAULT}
    k = api.tuning_key(model.step_args(), "f32_adaptive")
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    assert k.device.decode() == props.name and k.sm_count == props.multi_processor_count
    assert k.compute_capability == props.major * 10 + props.minor
    assert (k.nx, k.ny) == (model.layout.nx, model.layout.ny) and k.parts == 31 and k.warm_start == 0
    assert api.tuning_cache_find(path, k) is not None
    # another precision is another key: searched afresh
    third = model.autotune("f32", reps=1, cache=path)
    assert third["from_cache"] is False
    api.set_tuning(**DEFAULT)
