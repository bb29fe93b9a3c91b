"""Local machine-learned interatomic potentials (message passing over the GPU neighbour list).

Mirrors ``LocalMLIAPConfig`` / ``local_mliap_energy_full`` / ``local_mliap_energy_update``
(src/kups/potential/mliap/local.py:310-456): node embeddings h = init(Z), one message per
directed edge m_ij = edge(h_i, h_j, d_ij) with d_ij = x_j - x_i + s @ L, summed onto the
edge's first atom, per-atom energies readout(h, sum_j m_ij) summed per system.  The three
functions are the user's model and run as torch callables (the reference's are JAX
callables); the graph is ``kups_neighborlist_build`` on the device (the reference's full
directed neighbour list), and forces / cell gradients come from torch autograd through the
difference vectors (the reference's ``jax.vjp`` of the same expression).

The incremental path keeps the reference's cache (node embeddings and message sums) and
updates it for a set of changed atoms: messages of every edge touching a changed atom in the
old graph are subtracted, those of every such edge in the new graph added, and the readout
is evaluated again (local.py:359-421).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import torch

from .neighborlist import CellListNeighborList, NeighborListPoints


@dataclass
class LocalMLIAPCache:
    node_init: torch.Tensor  # [N, F]
    msg_sum: torch.Tensor  # [N, F']


@dataclass
class LocalMLIAPResult:
    energy: torch.Tensor  # [S]
    cache: LocalMLIAPCache
    grad: torch.Tensor | None = None  # dE/dx [N, 3]
    grad_tril: torch.Tensor | None = None  # dE/dtril [S, 6] at fixed Cartesian positions


def _segment_sum(values: torch.Tensor, index: torch.Tensor, n: int) -> torch.Tensor:
    out = torch.zeros((n,) + tuple(values.shape[1:]), dtype=values.dtype, device=values.device)
    return out.index_add(0, index.long(), values)


@dataclass
class LocalMLIAP:
    """init_function(Z [N]) -> [N, F]; edge_function(h_i, h_j, d [E, 3]) -> [E, F'];
    readout_function(h [N, F], msg_sum [N, F']) -> per-atom energies [N]."""

    init_function: Callable
    edge_function: Callable
    readout_function: Callable
    neighbor_list: CellListNeighborList = None

    def __post_init__(self):
        if self.neighbor_list is None:
            self.neighbor_list = CellListNeighborList(64)

    def graph(self, positions, system, tril, cutoffs):
        edges, self.neighbor_list = self.neighbor_list.call_and_fix(
            NeighborListPoints(positions.detach(), system), None, tril.detach(), cutoffs)
        return edges

    def _messages(self, h, edges, positions, system, tril):
        idx, _ = edges.valid()
        d = edges.difference_vectors(positions, system, tril)
        return self.edge_function(h[idx[:, 0].long()], h[idx[:, 1].long()], d), idx[:, 0]

    def energy(self, positions, atomic_numbers, system, tril, cutoffs, gradients: bool = True) -> LocalMLIAPResult:
        """local_mliap_energy_full, plus dE/dx and dE/dtril when ``gradients``."""
        pos = torch.as_tensor(positions, dtype=torch.float64, device="cuda")
        tr = torch.as_tensor(tril, dtype=torch.float64, device="cuda")
        sysi = torch.as_tensor(system, device="cuda").to(torch.int64)
        z = torch.as_tensor(atomic_numbers, device="cuda").to(torch.int64)
        edges = self.graph(pos, sysi, tr, cutoffs)
        if gradients:
            pos = pos.detach().requires_grad_(True)
            tr = tr.detach().requires_grad_(True)
        with torch.set_grad_enabled(gradients):
            h = self.init_function(z)
            m, first = self._messages(h, edges, pos, sysi, tr)
            msg = _segment_sum(m, first, pos.shape[0])
            e_atom = self.readout_function(h, msg)
            energy = _segment_sum(e_atom, sysi, tr.shape[0])
        grad = grad_tril = None
        if gradients:
            grad, grad_tril = torch.autograd.grad(energy.sum(), (pos, tr), allow_unused=True)
            grad = torch.zeros_like(pos) if grad is None else grad
            grad_tril = torch.zeros_like(tr) if grad_tril is None else grad_tril
        return LocalMLIAPResult(energy.detach(), LocalMLIAPCache(h.detach(), msg.detach()), grad, grad_tril)

    def energy_update(self, cache: LocalMLIAPCache, positions_old, positions_new, atomic_numbers_old,
                      atomic_numbers_new, changed, system, tril, cutoffs) -> LocalMLIAPResult:
        """local_mliap_energy_update: energies after replacing the positions / species of the
        atoms ``changed`` (all other atoms unchanged), from the cache of the old state."""
        tr = torch.as_tensor(tril, dtype=torch.float64, device="cuda")
        sysi = torch.as_tensor(system, device="cuda").to(torch.int64)
        old = torch.as_tensor(positions_old, dtype=torch.float64, device="cuda")
        new = torch.as_tensor(positions_new, dtype=torch.float64, device="cuda")
        z_new = torch.as_tensor(atomic_numbers_new, device="cuda").to(torch.int64)
        ch = torch.as_tensor(changed, device="cuda").to(torch.int64)
        n = old.shape[0]
        mask = torch.zeros(n, dtype=torch.bool, device="cuda")
        mask[ch] = True
        h_old = cache.node_init
        h_new = h_old.clone()
        h_new[ch] = self.init_function(z_new[ch]).to(h_old.dtype)
        msg = cache.msg_sum.clone()
        for h, pos, sign in ((h_old, old, -1.0), (h_new, new, 1.0)):
            edges = self.graph(pos, sysi, tr, cutoffs)
            idx, sh = edges.valid()
            touch = mask[idx[:, 0].long()] | mask[idx[:, 1].long()]
            sub = type(edges)(idx[touch].contiguous(), sh[touch].reshape(-1, 1, 3).contiguous(), int(touch.sum()))
            with torch.no_grad():
                m, first = self._messages(h, sub, pos, sysi, tr)
                msg = msg + sign * _segment_sum(m, first, n)
        with torch.no_grad():
            energy = _segment_sum(self.readout_function(h_new, msg), sysi, tr.shape[0])
        return LocalMLIAPResult(energy, LocalMLIAPCache(h_new, msg))
