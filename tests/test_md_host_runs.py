"""Runs of whole systems for the host-memory MD call (``md.run_bounds``, CPU): a particle table
grouped by system is cut at system boundaries into runs of about equal atom counts that
partition the atoms and the systems in order, each run holding atoms; any other table is one
run."""

import numpy as np
import pytest
import torch

from kups_gb300.md import run_bounds


def _system(counts):
    return torch.as_tensor(np.repeat(np.arange(len(counts)), counts), dtype=torch.int64)


def _check_partition(bounds, counts):
    n, s = int(sum(counts)), len(counts)
    assert bounds[0][0] == 0 and bounds[0][2] == 0 and bounds[-1][1] == n and bounds[-1][3] == s
    for (a0, a1, s0, s1), (b0, _, t0, _) in zip(bounds[:-1], bounds[1:]):
        assert a1 == b0 and s1 == t0
    for a0, a1, s0, s1 in bounds:
        assert a1 - a0 == sum(counts[s0:s1])
        if n > 0:
            assert a1 > a0


def test_uneven_counts_with_empty_systems():
    counts = [10, 0, 0, 5, 7, 0, 3]
    b = run_bounds(_system(counts), len(counts), 4)
    assert b == [(0, 10, 0, 1), (10, 15, 1, 4), (15, 22, 4, 5), (22, 25, 5, 7)]
    _check_partition(b, counts)


@pytest.mark.parametrize("chunks", [1, 2, 3, 4, 7])
def test_random_batches_partition_and_balance(chunks):
    rng = np.random.default_rng(chunks)
    counts = rng.integers(64, 2049, 300).tolist()
    b = run_bounds(_system(counts), len(counts), chunks)
    _check_partition(b, counts)
    assert len(b) == chunks
    sizes = [a1 - a0 for a0, a1, _, _ in b]
    assert max(sizes) - min(sizes) <= 2 * 2048  # within a system or two of equal


def test_degenerate_tables_are_one_run():
    assert run_bounds(torch.zeros(0, dtype=torch.int64), 3, 4) == [(0, 0, 0, 3)]
    assert run_bounds(_system([100]), 1, 4) == [(0, 100, 0, 1)]
    shuffled = _system([3, 4, 5])[torch.tensor([0, 5, 1, 9, 2, 3, 4, 6, 7, 8, 10, 11])]
    assert run_bounds(shuffled, 3, 4) == [(0, 12, 0, 3)]
    # fewer systems with atoms than runs asked for
    b = run_bounds(_system([0, 6, 0, 6]), 4, 4)
    _check_partition(b, [0, 6, 0, 6])
    assert len(b) == 2
