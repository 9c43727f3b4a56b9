"""Forcing time interpolation on the host: nesf_time_indices (the time indexing of a
FieldTimeSeries, which the atmosphere interpolation calls at interpolate_atmospheric_state.jl:
57-60) against the oracle's restatement, its known answers and its argument checks, and the
`.npy` snapshot source of the forcing window. No device work."""
import numpy as np
import pytest

from nesf import _lib
from nesf import forcing


def _cases(rng):
    uniform = np.arange(8) * 10800.0
    ragged = np.cumsum(rng.uniform(100.0, 5000.0, 20))
    return [uniform, ragged, np.array([0.0, 1.0]), np.array([5.0])]


@pytest.mark.parametrize("indexing", ["cyclical", "linear", "clamp"])
def test_time_indices_match_oracle(oracle, indexing):
    rng = np.random.default_rng(3)
    for times in _cases(rng):
        span = times[-1] - times[0] if len(times) > 1 else 1.0
        periods = (0.0,) if len(times) == 1 else (0.0, 1.5 * span + 10.0)
        for period in periods:
            ts = list(rng.uniform(times[0] - 3 * span, times[-1] + 3 * span, 300)) + list(times)
            ts += [times[-1] + 1e-3, times[0] - 1e-3, times[0] + 7 * (period or span)]
            for t in ts:
                got = forcing.time_indices(times, t, indexing, period)
                want = oracle.time_indices(times, indexing, period, t)
                assert got == want, (indexing, period, t)


def test_time_indices_known_answers():
    times = np.arange(8) * 10800.0          # a day of 3-hourly snapshots, cycled daily
    day = 86400.0
    assert forcing.time_indices(times, 0.0) == (0, 1, 0.0)
    assert forcing.time_indices(times, 5400.0) == (0, 1, 0.5)
    assert forcing.time_indices(times, 3 * 10800.0) == (3, 4, 0.0)
    assert forcing.time_indices(times, 7 * 10800.0 + 2700.0) == (7, 0, 0.25)   # the last blends into the first
    assert forcing.time_indices(times, day + 5400.0) == (0, 1, 0.5)           # one period later
    assert forcing.time_indices(times, -5400.0) == (7, 0, 0.5)                # one period earlier
    assert forcing.time_indices(times, -5400.0, "clamp") == (0, 0, 0.0)
    assert forcing.time_indices(times, 2 * day, "clamp") == (7, 7, 0.0)
    assert forcing.time_indices(times, -5400.0, "linear") == (0, 1, -0.5)     # extrapolated
    assert forcing.time_indices(times, 2 * day, "cyclical", period=2 * day) == (0, 1, 0.0)
    assert forcing.time_indices(np.array([5.0]), 123.0) == (0, 0, 0.0)


def test_time_indices_reject_bad_arguments():
    times = np.arange(8) * 10800.0
    with pytest.raises(_lib.NesfError):
        forcing.time_indices(times[::-1], 0.0)
    with pytest.raises(_lib.NesfError):
        forcing.time_indices(np.array([0.0, 1.0, 1.0]), 0.5)
    with pytest.raises(_lib.NesfError):
        forcing.time_indices(times, 0.0, "cyclical", period=times[-1] - times[0])   # not longer than the span
    with pytest.raises(_lib.NesfError):
        forcing.time_indices(times, float("nan"))


def test_npy_source_round_trip(tmp_path):
    rng = np.random.default_rng(4)
    arrays = {"u": rng.normal(size=(3, 6, 9)).astype(np.float32), "T": rng.normal(size=(3, 6, 9)).astype(np.float32)}
    forcing.NpySource.write(str(tmp_path), arrays)
    src = forcing.NpySource(str(tmp_path), arrays)
    out = np.empty((6, 9), np.float32)
    for name in arrays:
        for n in range(3):
            src.read(name, n, out)
            assert np.array_equal(out, arrays[name][n])
