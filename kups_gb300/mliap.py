"""Local machine-learned interatomic potentials (message passing over the GPU neighbour list).

Mirrors ``LocalMLIAPConfig`` / ``local_mliap_energy_full`` / ``local_mliap_energy_update``
(src/kups/potential/mliap/local.py:310-456): node embeddings h = init(Z), one message per
directed edge m_ij = edge(h_i, h_j, d_ij) with d_ij = x_j - x_i + s @ L, summed onto the
edge's first atom, per-atom energies readout(h, sum_j m_ij) summed per system.  The three
functions are the user's model and run as torch callables (the reference's are JAX
callables).  Everything around them is native: the graph (``kups_neighborlist_build``, the
reference's full directed neighbour list), the edge vectors (``kups_edge_vectors``), the
message sum (``kups_edge_segment_sum``, whose backward is the gather of the node gradient)
and the forces and cell gradient (``kups_edge_gradients`` from dE/dd_ij, the only gradient the
model's autograd is asked for: the reference's ``jax.vjp`` of the same expression).

The incremental path keeps the reference's cache (node embeddings and message sums) and
updates it for a set of changed atoms: messages of every edge touching a changed atom in the
old graph are subtracted, those of every such edge in the new graph added, and the readout
is evaluated again (local.py:359-421).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import torch

from . import _lib
from .neighborlist import CellListNeighborList, NeighborListPoints, _stream


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


def edge_vectors(positions, system, tril, edges) -> torch.Tensor:
    """d_e = x_j - x_i + s_e @ L of the valid edges, float64 [E, 3] (kups_edge_vectors)."""
    pos = positions.detach().to(torch.float64).contiguous()
    sysi = system.to(torch.int32).contiguous()
    tr = tril.detach().to(torch.float64).contiguous()
    ne = edges.n_edges
    d = torch.empty((ne, 3), dtype=torch.float64, device=pos.device)
    rc = _lib.load().kups_edge_vectors(pos.data_ptr(), sysi.data_ptr(), pos.shape[0], tr.data_ptr(), tr.shape[0],
                                       edges.indices.data_ptr(), edges.shifts.data_ptr(), ne, d.data_ptr(), _stream())
    _lib.check(rc, "kups_edge_vectors")
    return d


class _EdgeSegmentSum(torch.autograd.Function):
    """sum of edge rows onto the edge's first atom (kups_edge_segment_sum); backward: the node
    gradient gathered back to the edges."""

    @staticmethod
    def forward(ctx, values, edges_idx, n_edges, n):
        v = values.to(torch.float64).contiguous()
        w = int(v.shape[1]) if v.dim() > 1 else 1
        out = torch.empty((n, w), dtype=torch.float64, device=v.device)
        rc = _lib.load().kups_edge_segment_sum(v.data_ptr(), w, edges_idx.data_ptr(), n_edges, n, out.data_ptr(),
                                               _stream())
        _lib.check(rc, "kups_edge_segment_sum")
        ctx.save_for_backward(edges_idx)
        ctx.n_edges = n_edges
        ctx.shape = values.shape
        out = out.to(values.dtype)  # summed in float64, returned in the model's type
        return out if values.dim() > 1 else out[:, 0]

    @staticmethod
    def backward(ctx, grad_out):
        (edges_idx,) = ctx.saved_tensors
        first = edges_idx[: ctx.n_edges, 0].long()
        g = grad_out.index_select(0, first)
        return g.reshape(ctx.shape), None, None, None


def edge_gradients(dE_dd, system, n, n_systems, edges):
    """dE/dx [N, 3] and dE/dtril [S, 6] from dE/dd of the valid edges (kups_edge_gradients)."""
    g = dE_dd.detach().to(torch.float64).contiguous()
    sysi = system.to(torch.int32).contiguous()
    grad = torch.empty((n, 3), dtype=torch.float64, device=g.device)
    gt = torch.empty((n_systems, 6), dtype=torch.float64, device=g.device)
    rc = _lib.load().kups_edge_gradients(g.data_ptr(), sysi.data_ptr(), n, n_systems, edges.indices.data_ptr(),
                                         edges.shifts.data_ptr(), edges.n_edges, grad.data_ptr(), gt.data_ptr(),
                                         _stream())
    _lib.check(rc, "kups_edge_gradients")
    return grad, gt


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

    def _messages(self, h, edges, positions, system, tril, d=None):
        idx, _ = edges.valid()
        if d is None:
            d = edge_vectors(positions, system, tril, edges)
        return self.edge_function(h[idx[:, 0].long()], h[idx[:, 1].long()], d), idx[:, 0]

    def energy(self, positions, atomic_numbers, system, tril, cutoffs, gradients: bool = True) -> LocalMLIAPResult:
        """local_mliap_energy_full, plus dE/dx and dE/dtril when ``gradients``."""
        pos = torch.as_tensor(positions, dtype=torch.float64, device="cuda")
        tr = torch.as_tensor(tril, dtype=torch.float64, device="cuda")
        sysi = torch.as_tensor(system, device="cuda").to(torch.int64)
        z = torch.as_tensor(atomic_numbers, device="cuda").to(torch.int64)
        edges = self.graph(pos, sysi, tr, cutoffs)
        n, s = pos.shape[0], tr.shape[0]
        d = edge_vectors(pos, sysi, tr, edges)
        if gradients:
            d.requires_grad_(True)
        with torch.set_grad_enabled(gradients):
            h = self.init_function(z)
            m, _ = self._messages(h, edges, pos, sysi, tr, d)
            msg = _EdgeSegmentSum.apply(m, edges.indices, edges.n_edges, n)
            e_atom = self.readout_function(h, msg)
            energy = _segment_sum(e_atom, sysi, s)
        grad = grad_tril = None
        if gradients:
            (g_d,) = torch.autograd.grad(energy.sum(), (d,), allow_unused=True)
            g_d = torch.zeros_like(d) if g_d is None else g_d
            grad, grad_tril = edge_gradients(g_d, sysi, n, s, edges)
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
                m, _ = self._messages(h, sub, pos, sysi, tr)
                msg = msg + sign * _EdgeSegmentSum.apply(m, sub.indices, sub.n_edges, n).to(msg.dtype)
        with torch.no_grad():
            energy = _segment_sum(self.readout_function(h_new, msg), sysi, tr.shape[0])
        return LocalMLIAPResult(energy, LocalMLIAPCache(h_new, msg))
