"""The N > 1 path on CPU: two gloo ranks sharding independent units.

Each rank takes its share of the units (cost-balanced), computes them alone, and
rank 0 gathers and reassembles them; timings reduce by max.  The per-unit work
here is a host stand-in with a known answer (no GPU).
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from emerge_gb300.replicas import merge_by_index, partition


def test_partition_covers_and_balances():
    for world in (1, 2, 3, 8):
        parts = [partition(37, world, r) for r in range(world)]
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(37))
        rng = np.random.default_rng(world)
        costs = rng.uniform(1, 10, 37) ** 3          # uneven units (cavity sizes)
        parts = [partition(37, world, r, costs) for r in range(world)]
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(37))
        loads = np.array([costs[p].sum() for p in parts])
        assert loads.max() - loads.min() <= costs.max()          # greedy LPT bound
    with pytest.raises(ValueError):
        partition(5, 2, 2)


def test_merge_rejects_gaps_and_overlaps():
    with pytest.raises(ValueError):
        merge_by_index([(np.array([0, 1]), np.zeros(2)), (np.array([1, 2]), np.zeros(2))], 3)


def _unit(i):
    """A stand-in unit of work with a known result (an S-parameter-like 2x2 block)."""
    return np.array([[np.cos(i), np.sin(i)], [-np.sin(i), np.cos(i)]]) * (1 + 0.01j * i)


def _rank_main(rank, world, port, n_items, out_path):
    import torch.distributed as dist
    from emerge_gb300.replicas import gather_to_root, max_over_ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = 1.0 + np.arange(n_items) % 5
        mine = partition(n_items, world, rank, costs)
        vals = np.stack([_unit(int(i)) for i in mine])
        t = max_over_ranks(0.5 + rank)                  # each rank's "step time"
        parts = gather_to_root((mine, vals))
        if rank == 0:
            S = merge_by_index(parts, n_items)
            np.savez(out_path, S=S, t=t)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_shard_and_gather(tmp_path):
    n, world = 23, 2
    out = str(tmp_path / "res.npz")
    mp.start_processes(_rank_main, args=(world, _free_port(), n, out), nprocs=world, join=True,
                       start_method="spawn")
    z = np.load(out)
    assert float(z["t"]) == 1.5
    assert np.allclose(z["S"], np.stack([_unit(i) for i in range(n)]), rtol=0, atol=0)
