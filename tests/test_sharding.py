"""Data-parallel sharding of independent systems across ranks (CPU, gloo).

The partition is checked against brute force; two gloo ranks each take their
range of a batched LJ workload, evaluate it (the float64 oracle stands in for
the GPU kernel on this CPU-only path), and rank 0's gathered per-system
energies must equal the single-process result exactly.
"""

import itertools
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from kups_gb300.sharding import gather_per_system, partition_by_cost, rank_systems


def _brute(c, w):
    n = len(c)
    best = None
    for cuts in itertools.combinations_with_replacement(range(n + 1), w - 1):
        b = (0,) + cuts + (n,)
        if any(b[i] > b[i + 1] for i in range(w)):
            continue
        m = max(sum(c[b[i]:b[i + 1]]) for i in range(w))
        best = m if best is None else min(best, m)
    return best


@pytest.mark.parametrize("n,w", [(6, 2), (7, 3), (9, 4), (3, 5), (1, 1)])
def test_partition_is_contiguous_complete_and_optimal(n, w):
    c = np.random.default_rng(n * 10 + w).integers(1, 50, n).astype(float)
    r = partition_by_cost(c, w)
    assert len(r) == w and r[0][0] == 0 and r[-1][1] == n
    assert all(r[i][1] == r[i + 1][0] for i in range(w - 1))
    assert max(c[lo:hi].sum() for lo, hi in r) == pytest.approx(_brute(list(c), w))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system_energies(W, lo, hi):
    from oracle import md as omd

    sel = (W.system >= lo) & (W.system < hi)
    e, _, _ = omd.lj_forces(W.positions[sel], W.system[sel] - lo, W.species[sel], W.tril[lo:hi], W.sigma, W.epsilon,
                            np.full(hi - lo, W.cutoff))
    return e


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from kups_gb300 import workloads

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    W = workloads.batched_uneven_lj(n_systems=9, n_min=20, n_max=90, seed=4)
    counts = np.bincount(W.system, minlength=W.n_systems)
    ranges = [rank_systems(counts, r, world) for r in range(world)]
    lo, hi = ranges[rank]
    local = torch.as_tensor(_system_energies(W, lo, hi))
    gathered = gather_per_system(local, ranges, rank)
    if rank == 0:
        np.save(out_path, gathered.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_systems_and_gather(tmp_path):
    from kups_gb300 import workloads

    out = str(tmp_path / "gathered.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    W = workloads.batched_uneven_lj(n_systems=9, n_min=20, n_max=90, seed=4)
    expected = _system_energies(W, 0, W.n_systems)
    np.testing.assert_array_equal(np.load(out), expected)


def _system_stress(W, lo, hi):
    from oracle import md as omd

    sel = (W.system >= lo) & (W.system < hi)
    sysi = W.system[sel] - lo
    _, f, dt = omd.lj_forces(W.positions[sel], sysi, W.species[sel], W.tril[lo:hi], W.sigma, W.epsilon,
                             np.full(hi - lo, W.cutoff))
    return omd.virial_stress(W.positions[sel], -f, sysi, W.tril[lo:hi], dt)


def _rank_stress(rank, world, port, out_path):
    import torch.distributed as dist

    from kups_gb300 import workloads

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    W = workloads.batched_uneven_lj(n_systems=7, n_min=20, n_max=80, seed=6)
    counts = np.bincount(W.system, minlength=W.n_systems)
    ranges = [rank_systems(counts, r, world) for r in range(world)]
    lo, hi = ranges[rank]
    gathered = gather_per_system(torch.as_tensor(_system_stress(W, lo, hi)), ranges, rank)
    if rank == 0:
        np.save(out_path, gathered.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_per_system_stress_tensors(tmp_path):
    """Per-system [3, 3] observables (the virial stress of each rank's systems) gather in
    system order, trailing dimensions kept."""
    from kups_gb300 import workloads

    out = str(tmp_path / "stress.npy")
    mp.start_processes(_rank_stress, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    W = workloads.batched_uneven_lj(n_systems=7, n_min=20, n_max=80, seed=6)
    got = np.load(out)
    assert got.shape == (7, 3, 3)
    np.testing.assert_array_equal(got, _system_stress(W, 0, W.n_systems))
