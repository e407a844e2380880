"""Several GPUs: one process per GPU, launched by ``torch.distributed.run``.

The reference runs on one host and has no distributed path.  The scatter
estimate is a sum of independent z-slice terms (``Python/openSSS/
SingleScatterSimulationTOF.py:201``), so work splits by sampled z-slice (or
by whole problems / requests) with one sum of the compact sinograms at the
end and no exchange on the data path:

* ``partition_slices`` gives each rank a contiguous run of sampled slices
  with about the same number of scatter points;
* ``sharded_run`` runs a rank's slices and sums the ranks' leg-pair
  sinograms (``torch.distributed.all_reduce``);
* ``max_over_ranks`` is the bench's timing rule (the slowest rank).
"""

from __future__ import annotations

import os

import numpy as np


def rank_info() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def partition_slices(slice_counts, rank: int, world: int) -> tuple[int, int]:
    """Sampled z-slices [first, last) of ``rank``: contiguous runs that cover
    every slice exactly once, cut where the running point count crosses
    rank / world of the total."""
    counts = np.asarray(slice_counts, dtype=np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    cum = np.concatenate([[0], np.cumsum(counts)])
    total = cum[-1]
    cuts = [0] + [int(np.searchsorted(cum, total * k / world, side="left")) for k in range(1, world)] + [len(counts)]
    cuts = [min(max(c, 0), len(counts)) for c in cuts]
    for k in range(1, len(cuts)):
        cuts[k] = max(cuts[k], cuts[k - 1])
    return cuts[rank], cuts[rank + 1]


def max_over_ranks(value: float, device=None) -> float:
    """The largest ``value`` over the ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(t):
    """In-place sum of a tensor over the ranks of the default process group."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t)
    return t


def sharded_run(engine, ActivityMap, AttenuationMap, ImageSize, rank: int, world: int):
    """This rank's share of one simulation, summed over the ranks: every rank
    returns the full leg-pair sinogram [B, NL, NL] (CUDA)."""
    from .engine import fortran_flat

    dev = engine.device
    shape = tuple(int(s) for s in np.shape(ActivityMap))
    act = fortran_flat(ActivityMap, dev)
    mu = fortran_flat(AttenuationMap, dev)
    _, counts = engine.scatter_points(engine.problem(act, mu, shape, ImageSize))
    first, last = partition_slices(counts, rank, world)
    out = engine.run_flat(act, mu, shape, ImageSize, slice_range=(first, last))
    return sum_over_ranks(out)
