"""One process per GPU, independent units: the multi-GPU layer of this package.

The frequency-domain path shards without a data-path collective: sweep
frequency points, eigen instances and whole assemblies are independent units.
Each rank takes its share (``partition``), works alone on its own GPU, and the
host gathers the small results (S-parameters, eigenvalues, timings) on rank 0
(``gather_to_root``). The only collectives are these host-side gathers and the
max-over-ranks of a timing (``max_over_ranks``), on whatever process group is
initialised: NCCL between GPUs, gloo on CPU.
"""
from __future__ import annotations

import numpy as np


def partition(n_items: int, world: int, rank: int, costs=None) -> np.ndarray:
    """Indices of the items rank ``rank`` handles, in ascending order.

    Without costs: round-robin (item i to rank i % world).  With costs: greedy
    longest-processing-time, heaviest item first to the least-loaded rank (ties to
    the lower rank), so ranks finish together on uneven units such as cavities of
    different sizes.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if costs is None:
        return np.arange(rank, n_items, world, dtype=np.int64)
    c = np.asarray(costs, dtype=float)
    if c.shape != (n_items,):
        raise ValueError("one cost per item")
    load = np.zeros(world)
    owner = np.empty(n_items, dtype=np.int64)
    for i in np.argsort(-c, kind="stable"):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += c[i]
    return np.flatnonzero(owner == rank).astype(np.int64)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(x: float, device=None) -> float:
    """The maximum of ``x`` over all ranks (``x`` itself without a process group)."""
    dist = _dist()
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_root(obj):
    """Every rank's ``obj`` as a list on rank 0 (rank order), None elsewhere."""
    dist = _dist()
    if dist is None:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def merge_by_index(parts, n_items: int):
    """Reassemble per-rank results: ``parts`` = [(indices, values), ...] with values
    indexed like indices along axis 0; returns the values of all items in order."""
    idx = np.concatenate([np.asarray(i, dtype=np.int64) for i, _ in parts])
    if idx.size != n_items or not np.array_equal(np.sort(idx), np.arange(n_items)):
        raise ValueError("the parts do not cover every item exactly once")
    vals = np.concatenate([np.asarray(v) for _, v in parts], axis=0)
    out = np.empty_like(vals)
    out[idx] = vals
    return out
