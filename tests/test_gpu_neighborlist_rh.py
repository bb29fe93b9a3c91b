"""GPU neighbour list with a separate rh table and the Monte Carlo edge changes, against the oracle.

Bars: bit-exact sorted (i, j, shift) rows, duplicates included, for
* rh subsets without a remap (edges lh -> rh) on random triclinic batches whose cutoffs need
  periodic images, with exclusion and inclusion labels (src/kups/core/neighborlist.py:226-255,
  505-740);
* rh subsets with rh_index_remap (both directions, the i >= remap[j] rule);
* neighborlist_changes (:1425-1515): added / removed edges of moving k particles, equal to the
  oracle's and to the two separate rh calls after and before the move (the reference's own
  test, test/core/test_neighborlist.py:1553-1605).
"""

import numpy as np
import pytest
import torch

from oracle import neighborlist as onl

from test_gpu_core import random_triclinic_batch

pytestmark = pytest.mark.gpu


def cuda(x, dtype):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


def pts(pos, sysi, incl=None, excl=None, n_incl=None):
    from kups_gb300.neighborlist import NeighborListPoints

    return NeighborListPoints(cuda(pos, torch.float64), cuda(sysi, torch.int32),
                              None if incl is None else cuda(incl, torch.int32),
                              None if excl is None else cuda(excl, torch.int32), n_incl)


def rows(edges):
    i, s = edges.valid()
    return onl.sort_edges(i.cpu().numpy(), s.cpu().numpy())


def same(got, exp):
    assert got[0].shape == exp[0].shape, (got[0].shape, exp[0].shape)
    np.testing.assert_array_equal(got[0], exp[0])
    np.testing.assert_array_equal(got[1], exp[1])


def _rh_subset(seed, n_rh):
    pos, sysi, tril, cut, excl, incl = random_triclinic_batch(seed, n_sys=5)
    rng = np.random.default_rng(seed + 100)
    j = rng.choice(len(pos), n_rh, replace=False)
    rpos = pos[j] + rng.normal(0, 0.7, (n_rh, 3))
    return pos, sysi, tril, cut, excl, incl, j, rpos


@pytest.mark.parametrize("seed", [0, 1])
def test_rh_subset_without_remap(seed):
    from kups_gb300.neighborlist import CellListNeighborList

    pos, sysi, tril, cut, excl, incl, j, rpos = _rh_subset(seed, 40)
    rexcl = excl[j]  # the moved copies share their molecule's label
    exp = onl.neighbor_list_rh(pos, sysi, rpos, sysi[j], tril, cut, lh_inclusion=incl, rh_inclusion=incl[j],
                               lh_exclusion=excl, rh_exclusion=rexcl, n_inclusion=len(tril))
    edges, _ = CellListNeighborList(8).call_and_fix(pts(pos, sysi, incl, excl, len(tril)),
                                                     pts(rpos, sysi[j], incl[j], rexcl), cuda(tril, torch.float64),
                                                     cuda(cut, torch.float64))
    assert len(exp[0]) > 0
    same(rows(edges), exp)


@pytest.mark.parametrize("seed", [2, 3])
def test_rh_subset_with_remap(seed):
    from kups_gb300.neighborlist import CellListNeighborList

    pos, sysi, tril, cut, excl, incl, j, rpos = _rh_subset(seed, 25)
    exp = onl.neighbor_list_rh(pos, sysi, rpos, sysi[j], tril, cut, lh_inclusion=incl, rh_inclusion=incl[j],
                               lh_exclusion=excl, rh_exclusion=excl[j], rh_index_remap=j, n_inclusion=len(tril))
    edges, _ = CellListNeighborList(8).call_and_fix(pts(pos, sysi, incl, excl, len(tril)),
                                                     pts(rpos, sysi[j], incl[j], excl[j]), cuda(tril, torch.float64),
                                                     cuda(cut, torch.float64), cuda(j, torch.int32))
    assert len(exp[0]) > 0
    same(rows(edges), exp)


@pytest.mark.parametrize("n,m,seed,rc", [(10, 3, 42, 3.0), (30, 5, 123, 3.0), (200, 9, 5, 6.0)])
def test_neighborlist_changes_match_oracle_and_separate_calls(n, m, seed, rc):
    from kups_gb300.neighborlist import CellListNeighborList, neighborlist_changes

    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 9, (n, 3))
    changed = rng.choice(n, m, replace=False)
    new = rng.uniform(0, 9, (m, 3))
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0]])
    batch = np.zeros(n, int)
    nl = CellListNeighborList(16)
    res = neighborlist_changes(nl, pts(pos, batch), cuda(changed, torch.int32), pts(new, batch[changed]),
                               cuda(tril, torch.float64), cuda([rc], torch.float64))
    exp_a, exp_r = onl.neighborlist_changes(pos, batch, changed, new, tril, [rc])
    same(rows(res.added), exp_a)
    same(rows(res.removed), exp_r)
    # the two separate rh calls, after and before
    after = pos.copy()
    after[changed] = new
    a, _ = nl.call_and_fix(pts(after, batch), pts(new, batch[changed], None, changed), cuda(tril, torch.float64),
                           cuda([rc], torch.float64), cuda(changed, torch.int32))
    r, _ = nl.call_and_fix(pts(pos, batch), pts(pos[changed], batch[changed], None, changed),
                           cuda(tril, torch.float64), cuda([rc], torch.float64), cuda(changed, torch.int32))
    same(rows(res.added), rows(a))
    same(rows(res.removed), rows(r))


@pytest.mark.parametrize("compaction", [0.5, 0.75, 1.0])
def test_neighborlist_changes_single_particle_known_answer(compaction):
    """test/core/test_neighborlist.py:1607-1640, 1672-1700."""
    from kups_gb300.neighborlist import CellListNeighborList, neighborlist_changes

    pos = np.array([[0.0, 0, 0], [1.0, 0, 0], [5.0, 0, 0]])
    batch = np.zeros(3, int)
    res = neighborlist_changes(CellListNeighborList(8), pts(pos, batch), cuda([1], torch.int32),
                               pts([[4.5, 0, 0]], [0]), cuda([[10.0, 0, 10.0, 0, 0, 10.0]], torch.float64),
                               cuda([1.5], torch.float64), compaction=compaction)
    added = {tuple(map(int, r)) for r in rows(res.added)[0]}
    removed = {tuple(map(int, r)) for r in rows(res.removed)[0]}
    assert {(0, 1), (1, 0)} <= removed and (1, 2) not in removed
    assert {(1, 2), (2, 1)} <= added and (0, 1) not in added
