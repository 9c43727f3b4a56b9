"""Sharding of the interface-flux step over ranks (one process per GPU).

The step's cells are independent: the exchange grid splits into latitude bands
(`band`), each rank solving its own band with no exchange of fields (the fluxes
are computed into the one-cell halo ring, so a band needs only its own rows; the
interpolation reads a one-row overlap of the coarse atmosphere grid, which every
rank holds whole). The one collective is the final reduction of the FP64
compensated global integrals (nesf_area_integrals returns (sum, residual) pairs):
`reduce_integral_pairs` gathers every rank's pairs and combines them with
error-free two-sums in rank order, so every rank gets the same pair, and its sum is
the correctly rounded total of all ranks' cell terms, whatever the banding.
"""
import numpy as np


def band(ny, rank, world):
    """Rows [j0, j1) (0-based, interior) of `rank`'s latitude band: `world` bands of
    nearly equal height, the first `ny % world` one row taller."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    base, extra = divmod(ny, world)
    j0 = rank * base + min(rank, extra)
    return j0, j0 + base + (1 if rank < extra else 0)


def two_sum(a, b):
    """Knuth's error-free sum: s + e == a + b exactly (round to nearest)."""
    s = a + b
    bb = s - a
    e = (a - (s - bb)) + (b - bb)
    return s, e


def combine_pairs(pairs):
    """Sum (sum, residual) pairs, one row per integral, in the given order, as an
    unevaluated pair: the first element is the correctly rounded total whenever the
    residuals stay below half an ulp of it (they do for the pairs of
    nesf_area_integrals, whose residuals are the rounding errors of their sums)."""
    pairs = np.asarray(pairs, dtype=np.float64)          # (ranks, n, 2)
    out = np.zeros(pairs.shape[1:], dtype=np.float64)
    for k in range(pairs.shape[1]):
        hi, lo = 0.0, 0.0
        for r in range(pairs.shape[0]):
            for x in pairs[r, k]:
                hi, e = two_sum(hi, float(x))
                lo += e
        hi, lo = two_sum(hi, lo)
        out[k] = (hi, lo)
    return out


def reduce_integral_pairs(pairs, group=None):
    """All-gather each rank's (n, 2) integral pairs (torch.distributed, any backend) and
    combine them in rank order: the same (n, 2) result on every rank."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    local = torch.as_tensor(np.asarray(pairs, dtype=np.float64))
    device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    local = local.to(device)
    gathered = [torch.empty_like(local) for _ in range(world)]
    dist.all_gather(gathered, local, group=group)
    return combine_pairs(np.stack([g.cpu().numpy() for g in gathered]))
