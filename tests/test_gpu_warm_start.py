"""The learned warm start end to end: solver-generated samples, training on the tensor
cores, and the adaptive FP32 solver started from the network's guesses -- fewer
iterations for the same answer (within 1e-5 of the oracle, like the cold start)."""
import numpy as np
import pytest

from helpers import rel_err, widen
from nesf import api
from nesf import fields as F
from nesf import params as P
from nesf import synthetic as syn
from nesf import warm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    spec = P.atmosphere_ocean_interface_spec()
    # the widened open-ocean states, and coupled states like the workload's (open water in the
    # ice band, where the air is far colder than the ocean)
    states = [syn.warm_training_state(seed=300 + k, nx=360, ny=180) for k in range(4)]
    states += [syn.coupled(seed=500 + k, nx=360, ny=180, lat_s=-80, lat_n=80, land=0.3, interpolate=False)
               for k in range(3)]
    x, t = warm.training_set(spec, states)
    assert x.shape[0] > 250000
    net = warm.WarmStartNetwork(seed=7)
    net.fit_normalization(x, t)
    losses = []
    for epochs, lr in ((12, 2e-3), (8, 5e-4), (5, 1e-4)):    # a step-decayed learning rate
        losses += net.train(x, t, epochs=epochs, batch=2048, lr=lr)
    return spec, net, losses


def solve(spec, st, mlp=None):
    import torch
    dev = api.to_device({k: st.fields.get(k) for k in F.AO_INPUTS if k in st.fields})
    out = {k: torch.zeros(st.layout.shape, dtype=dev["u_atm"].dtype, device="cuda") for k in F.AO_OUTPUTS}
    stats = api.compute_atmosphere_ocean_fluxes(spec, st.layout, dev, out, precision="f32_adaptive", stats=True,
                                                mlp=mlp)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}, stats


def test_training_converges(trained):
    _, net, losses = trained
    assert losses[-1] < 0.03 * losses[0], " ".join(f"{v:.4f}" for v in losses)


def test_warm_start_cuts_iterations_at_the_same_accuracy(trained, oracle):
    spec, net, _ = trained
    st = syn.coupled(seed=401, nx=240, ny=120, lat_s=-75, lat_n=75, land=0.3, interpolate=False)
    ref = oracle.ao_fluxes(spec.to_c(), st.layout, widen(st.fields))
    cold, s_cold = solve(spec, st)
    hot, s_hot = solve(spec, st, mlp=net)
    R = st.layout.ring
    for k in F.AO_OUTPUTS:
        e = rel_err(R(hot[k]).astype(np.float64), R(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-5, (k, e.max())
    assert s_hot["solved"] == s_cold["solved"]
    per_cold = s_cold["iterations"] / s_cold["solved"]
    per_hot = s_hot["iterations"] / s_hot["solved"]
    assert per_hot < 0.85 * per_cold, (per_hot, per_cold)
    # the residual test sends back the cells whose guess is worse than 10x the cold start's first
    # residual -- mostly strongly stable cells, whose cold first iterate barely moves
    assert s_hot["cold_fallbacks"] < 0.15 * s_hot["solved"], (s_hot["cold_fallbacks"], s_hot["solved"])


def test_untrained_network_stays_exact(oracle):
    """A network that has not been trained guesses badly; the iteration still runs to the
    reference's tolerance from there, and the answer is unchanged."""
    spec = P.atmosphere_ocean_interface_spec()
    net = warm.WarmStartNetwork(seed=11)
    st = syn.coupled(seed=402, nx=120, ny=60, lat_s=-70, lat_n=70, land=0.2, interpolate=False)
    ref = oracle.ao_fluxes(spec.to_c(), st.layout, widen(st.fields))
    hot, s_hot = solve(spec, st, mlp=net)
    R = st.layout.ring
    for k in ("latent_heat", "sensible_heat", "x_momentum"):
        e = rel_err(R(hot[k]).astype(np.float64), R(ref[k]), floor_frac=1e-6)
        assert e.max() <= 1e-5, (k, e.max())
    assert s_hot["solved"] > 0 and s_hot["nonconverged"] == 0
