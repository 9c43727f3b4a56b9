"""The fused coupling step (nesf_coupling_step) and its CUDA graph (nesf_graph_*), through
the C ABI: the same kernels in update_state!'s order, so the outputs are bit-identical to
the per-phase entry points', and a replayed graph reproduces a direct step, including
after its time weight is changed."""
import numpy as np
import pytest

from helpers import to_numpy
from nesf import fields as F
from nesf import synthetic as syn
from nesf.coupled import CoupledModel, ICE_NET, OCEAN_NET, RAD_DIAG

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    st = syn.coupled(seed=41, nx=240, ny=120, lat_s=-80, lat_n=80, land=0.3, interpolate=True)
    return CoupledModel(st)


def outputs(m):
    import torch
    torch.cuda.synchronize()
    out = {("ao", k): to_numpy(m.ao[k]).copy() for k in F.AO_OUTPUTS}
    out.update({("ai", k): to_numpy(m.ai[k]).copy() for k in F.AI_OUTPUTS})
    out[("ai", "interface_temperature")] = to_numpy(m.ai["interface_temperature"]).copy()
    out.update({("io", k): to_numpy(m.io[k]).copy() for k in F.IO_OUTPUTS})
    out.update({("net", k): to_numpy(m.net[k]).copy() for k in OCEAN_NET + ICE_NET + RAD_DIAG})
    out[("x", "T_oc")] = to_numpy(m.x["T_oc"]).copy()
    out[("x", "T_atm")] = to_numpy(m.x["T_atm"]).copy()
    return out


def assert_same(a, b, label):
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), (label, k)


@pytest.mark.parametrize("precision", ["f64", "f32_adaptive"])
def test_native_step_matches_phase_calls(model, precision):
    model.reset()
    model.update_state(precision)
    ref = outputs(model)
    model.reset()
    model.native_step(precision)
    assert_same(ref, outputs(model), precision)
    assert np.isfinite(ref[("net", "ocean_T")]).all()


def test_graph_replays_the_step(model):
    model.reset()
    model.native_step("f32_adaptive")
    ref = outputs(model)
    model.capture("f32_adaptive")
    for _ in range(2):   # replayed twice from the same state
        model.reset()
        model.graph_step()
        assert_same(ref, outputs(model), "graph")


def test_graph_time_weight_update(model):
    step = model.step_args()
    tn0 = model.atmos["time_weight"]
    model.reset()
    step.set_time_weight(0.25)
    model.native_step("f32_adaptive")
    ref = outputs(model)
    step.set_time_weight(tn0)
    model.capture("f32_adaptive")
    model.reset()
    model.graph_step(time_weight=0.25)
    got = outputs(model)
    assert_same(ref, got, "time weight")
    model.reset()
    model.graph_step(time_weight=tn0)
    assert not np.array_equal(outputs(model)[("x", "T_atm")], got[("x", "T_atm")])


def test_graph_rejects_bad_weight(model):
    from nesf import _lib
    model.capture("f32_adaptive")
    with pytest.raises(_lib.NesfError):
        model.graph.set_time_weight(1.5)


def test_graph_with_warm_start_network(model):
    """A captured step that starts its FP32 solves from a network (here untrained: the
    fallback keeps the answers) replays like the direct step."""
    from nesf.warm import WarmStartNetwork
    model.mlp = WarmStartNetwork(seed=2)
    try:
        model.reset()
        model.native_step("f32_adaptive")
        ref = outputs(model)
        model.capture("f32_adaptive")
        model.reset()
        model.graph_step()
        assert_same(ref, outputs(model), "warm graph")
    finally:
        model.mlp = None
