"""The sharded step's host logic with world_size 2 on CPU (gloo): latitude bands cover the
grid once, and the cross-rank reduction of compensated integral pairs gives every rank the
same pair, whose sum is the correctly rounded total of all cells (the reference's
conservation integrals, test_conservation.jl:100-101), for any banding."""
import os
from fractions import Fraction

import numpy as np
import pytest
import torch.multiprocessing as mp

from nesf import distributed as D


def _pairs_of(x):
    """(sum, residual) of a rank's cell terms by the same compensated summation."""
    hi, lo = 0.0, 0.0
    for t in x.ravel():
        hi, e = D.two_sum(hi, float(t))
        lo += e
    return D.two_sum(hi, lo)


def _field(ny=37, nx=50, seed=3):
    rng = np.random.default_rng(seed)
    # terms of very different sizes and signs, as net heat fluxes times cell areas are
    return rng.normal(0, 1, (ny, nx)) * 10.0 ** rng.integers(-8, 9, (ny, nx))


def test_bands_cover_the_grid():
    for ny in (1, 7, 1280):
        for world in (1, 2, 3, 8):
            rows = [D.band(ny, r, world) for r in range(world)]
            assert rows[0][0] == 0 and rows[-1][1] == ny
            assert all(a[1] == b[0] for a, b in zip(rows, rows[1:]))
            h = [j1 - j0 for j0, j1 in rows]
            assert max(h) - min(h) <= 1
    with pytest.raises(ValueError):
        D.band(10, 2, 2)


def test_combine_pairs_is_correctly_rounded():
    x = _field()
    exact = float(sum((Fraction(float(t)) for t in x.ravel()), Fraction(0)))
    for world in (1, 2, 5):
        parts = [x[slice(*D.band(x.shape[0], r, world))] for r in range(world)]
        pairs = np.array([[_pairs_of(p)] for p in parts])        # (world, 1, 2)
        hi, lo = D.combine_pairs(pairs)[0]
        assert hi == exact, world


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x = _field()
        j0, j1 = D.band(x.shape[0], rank, world)
        y = x[j0:j1]
        local = np.array([_pairs_of(y), _pairs_of(y * y)])       # two integrals
        res = D.reduce_integral_pairs(local)
        out[rank] = res.tolist()
    finally:
        dist.destroy_process_group()


def test_gloo_world_size_2_reduction():
    x = _field()
    exact = [float(sum((Fraction(float(t)) for t in v.ravel()), Fraction(0))) for v in (x, x * x)]
    port = 29600 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = [np.array(out[r]) for r in range(2)]
    assert np.array_equal(res[0], res[1])                          # every rank gets the same pairs
    assert [r[0] for r in res[0]] == exact                        # correctly rounded totals
