"""Kernel-boundary tracing of the coupling step (nesf_trace_enable / nesf_trace_read):
the marks of a direct step and of a graph replay name every kernel phase, advance on
each stream, and end within the step."""
import pytest

from nesf import api
from nesf import synthetic as syn
from nesf.coupled import CoupledModel

pytestmark = pytest.mark.gpu

EXPECTED = {"step", "interpolate", "ai_classify", "ai_pass1", "ai_polish", "ai_replay", "ai_polish_replay",
            "sea_ice_ocean_fluxes", "ao_classify", "ao_pass1", "ao_polish", "ao_replay", "frazil_adjustment",
            "assembly"}


@pytest.fixture(scope="module")
def model():
    st = syn.coupled(seed=45, nx=240, ny=120, lat_s=-80, lat_n=80, land=0.3, interpolate=True)
    m = CoupledModel(st)
    api.trace_enable(True)
    yield m
    api.trace_enable(False)


def check_marks(marks):
    import torch
    names = {n for n, _, _ in marks}
    assert EXPECTED <= names, EXPECTED - names
    assert marks[0][0] == "step" and marks[0][2] == 0.0
    last = {}
    for name, stream, t in marks:
        assert t >= last.get(stream, 0.0) - 1e-3, (name, stream, t)
        last[stream] = t
    assert len({s for _, s, _ in marks}) >= 3       # the caller's stream, the sea-ice lane, its replay lane
    spans = api.timeline(marks)
    assert all(e >= 0 for _, _, _, e in spans)


def test_direct_step_marks(model):
    import torch
    model.reset()
    model.native_step("f32_adaptive")
    torch.cuda.synchronize()
    check_marks(api.trace_read())


def test_graph_replay_marks(model):
    import torch
    model.capture("f32_adaptive")
    model.reset()
    model.graph_step()
    torch.cuda.synchronize()
    check_marks(api.trace_read())
