"""The oracle's coupling step on a band of rows equals the same rows of the whole grid.

The config-size GPU tests and the bench's error statistics compare the GPU step with
the oracle on sampled bands of rows (the oracle is too slow for the whole 1/8-degree
grid). That is only valid if every phase is per cell up to its neighbour reads, so a
band with its halos reproduces the whole-grid answer exactly on its interior; this
test checks it bit for bit on a small coupled workload with interpolation, land and
sea ice, for bands in the middle and at both edges of the grid.
"""
import numpy as np
import pytest

from nesf import params as P
from nesf import synthetic as syn


@pytest.fixture(scope="module")
def workload():
    return syn.coupled(seed=77, nx=48, ny=40, lat_s=-80, lat_n=80, land=0.3, interpolate=True, dtype=np.float32)


def specs():
    return dict(ao_spec=P.atmosphere_ocean_interface_spec(), ai_spec=P.atmosphere_sea_ice_interface_spec(),
                io_spec=P.SeaIceOceanSpec(), asm_spec=P.AssemblySpec())


@pytest.mark.parametrize("lo,rows", [(0, 6), (13, 8), (34, 6)])
def test_band_equals_whole_grid_rows(workload, lo, rows):
    from oracle import band as OB
    st = workload
    L = st.layout
    full_layout, full = OB.step_band(st, 0, L.ny, **specs())
    sub, part = OB.step_band(st, lo, rows, **specs())
    assert set(part) == {"atmos", "ao", "ai", "io", "net", "inputs"}
    for group in ("atmos", "ao", "ai", "io", "net"):
        for k, v in part[group].items():
            if k == "T_oc":
                v, w = v[0], full[group][k][0]
            else:
                w = full[group][k]
            got = sub.interior(v)
            want = full_layout.interior(w)[lo:lo + rows]
            assert np.array_equal(got, want), (group, k)
    # the band holds ice, land and water cells
    band_ice = sub.interior(OB.band_of(st.fields["ice_concentration"], st, lo, rows)) > 0
    assert band_ice.any() or lo == 13


def test_error_table_floor_and_exclusion():
    from oracle import band as OB
    t = OB.ErrorTable()
    ref = np.array([1.0, 2.0, 1e-9, 4.0])
    got = np.array([1.0 + 1e-6, 2.0, 1e-9 + 1e-12, 5.0])
    t.add("x", got, ref, keep=np.array([True, True, True, False]))
    s = t.summary()["x"]
    assert s["cells"] == 3
    # the near-zero cell is compared on the floor 1e-6 * max|ref| = 2e-6 (error 5e-7), so
    # the first cell's 1e-6 is the largest
    assert abs(s["max"] - 1e-6) < 1e-12
