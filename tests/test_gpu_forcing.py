"""The forcing window (nesf/forcing.py) on the GPU: snapshots streamed from `.npy` files into
K device slots, the pair of each time handed to nesf_interpolate_atmosphere_state through the
snapshot stride, against the interpolation of the same pair passed explicitly: identical
outputs over more than two cycles, including the pair that wraps from the last snapshot to
the first (11 snapshots in 5 slots: with slot = index mod 5 both would share a slot)."""
import numpy as np
import pytest

from helpers import to_numpy
from nesf import api
from nesf import forcing
from nesf import synthetic as syn

pytestmark = pytest.mark.gpu


def test_window_interpolation_matches_explicit_pairs(oracle, tmp_path):
    import torch
    rng = np.random.default_rng(11)
    nt, dt = 11, 10800.0
    at = syn._coarse_atmosphere(rng, nxa=64, nya=32, nt=nt)
    times = np.arange(nt) * dt
    forcing.NpySource.write(str(tmp_path), at["arrays"])
    src = forcing.NpySource(str(tmp_path), at["arrays"])
    L = syn.Layout(120, 50, 3, 3)
    coords = syn.lonlat(120, 50, -75.0, 75.0)
    win = forcing.FieldTimeSeriesWindow(src, times, at["layout"], slots=5)
    period = nt * dt
    ts = list(np.linspace(-period, 2.2 * period, 41)) + [times[3], times[-1], times[-1] + dt / 2, period]
    try:
        for t in ts:
            arrays, stride, w = win.update(t)
            out = {n: torch.zeros(L.shape, dtype=torch.float32, device="cuda") for n in arrays}
            api.interpolate_atmosphere_state(L, coords, dict(at, stride_t=stride), arrays, out, w)
            win.release()
            n1, n2, w_ref = oracle.time_indices(times, "cyclical", 0.0, t)
            pair = {n: torch.tensor(np.stack([at["arrays"][n][n1], at["arrays"][n][n2]]), device="cuda")
                    for n in arrays}
            ref = {n: torch.zeros_like(out[n]) for n in arrays}
            api.interpolate_atmosphere_state(L, coords, at, pair, ref, w_ref)
            torch.cuda.synchronize()
            assert w == w_ref
            for n in arrays:
                assert torch.equal(out[n], ref[n]), (t, n)
        assert win.uploads < 2 * len(ts)   # the window reuses and prefetches its slots
    finally:
        win.close()


def test_graph_follows_the_window(tmp_path):
    """A captured coupling step fed by the window through nesf_graph_set_forcing: after each
    replay the exchange-grid atmosphere equals the interpolation of the explicit pair."""
    import torch
    from nesf.coupled import ATMOS_NAMES, EXCHANGE_ATMOS, CoupledModel
    st = syn.coupled(seed=21, nx=240, ny=120, lat_s=-80, lat_n=80, land=0.3, interpolate=True)
    base = st.atmos["arrays"]
    nt, dt = 7, 10800.0
    series = {n: np.stack([base[n][k % 2] * (1 + 0.01 * k) if n not in ("u", "v") else base[n][k % 2] + 0.3 * k
                           for k in range(nt)]).astype(base[n].dtype) for n in base}
    times = np.arange(nt) * dt
    m = CoupledModel(st)
    m.capture("f32_adaptive")
    caches = m.fractional_indices()   # the direct call interpolates with the caches (the gather kernel)
    dtype = torch.from_numpy(series["T"][:1]).dtype
    win = forcing.FieldTimeSeriesWindow(forcing.ArraySource(series), times, st.atmos["layout"], slots=3, dtype=dtype)
    try:
        for t in (0.0, 0.4 * dt, 2.5 * dt, 6.5 * dt, 7.25 * dt, 13.0 * dt):
            arrays, stride, w = win.update(t)
            m.graph.set_forcing(arrays, stride, w)
            m.reset()
            m.graph_step()
            win.release()
            n1, n2, _ = forcing.time_indices(times, t)
            pair = {n: torch.tensor(np.stack([series[n][n1], series[n][n2]]), device="cuda") for n in series}
            ref = {n: torch.zeros_like(m.x[EXCHANGE_ATMOS[n]]) for n in ATMOS_NAMES}
            api.interpolate_atmosphere_state(m.layout, m.coords, st.atmos, pair, ref, w, frac=caches)
            torch.cuda.synchronize()
            R = m.layout.ring   # the interpolation writes the interior and its one-cell ring
            for n in ATMOS_NAMES:
                assert np.array_equal(R(to_numpy(m.x[EXCHANGE_ATMOS[n]])), R(to_numpy(ref[n]))), (t, n)
            assert torch.isfinite(m.ao["latent_heat"]).all()
    finally:
        win.close()
        m.graph.close()
