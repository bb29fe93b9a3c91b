"""Lennard-Jones potential on the GPU behind kUPS's ``Potential`` interface.

Mirrors src/kups/core/potential.py (``PotentialOut`` :78-139, ``Potential``
:142-198) and src/kups/potential/classical/lennard_jones.py
(``LennardJonesParameters`` :82-141, ``make_lennard_jones_potential``
:355-392).  The energy and both gradients (positions and cell ``tril``, the
``PositionAndUnitCell`` pair of src/kups/potential/common/energy.py:57-59)
come from the ``kups_lj_edges`` CUDA kernel over the GPU neighbour list.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, NamedTuple

import torch

from . import _lib
from .neighborlist import CellListNeighborList, NeighborListPoints, _f64, _i32, _stream, new_status, read_status
from .unitcell import as_tril


class PositionAndUnitCell(NamedTuple):
    positions: torch.Tensor  # dE/dx [N, 3]
    unitcell: torch.Tensor  # dE/dtril [S, 6]


@dataclass
class PotentialOut:
    total_energies: torch.Tensor  # [S]
    gradients: Any = None
    hessians: Any = None
    cache: Any = None  # what a later patched call starts from (``CachedPotential``'s cached value)


@dataclass
class ParticlePatch:
    """Particles ``indices`` take ``positions`` (the ``ParticlePositionChanges`` a Monte Carlo move
    proposes, src/kups/mcmc/moves.py:222-295; applied as a patch, src/kups/core/patch.py:37-49)."""

    indices: torch.Tensor  # int [k], distinct
    positions: torch.Tensor  # f64 [k, 3]


def patched_positions(positions: torch.Tensor, patch: ParticlePatch) -> torch.Tensor:
    new = _f64(positions).clone()
    new[_i32(patch.indices).long()] = _f64(patch.positions)
    return new


def changed_edges(neighborlist, positions, system, inclusion, exclusion, tril, cutoffs, patch: ParticlePatch):
    """(added, removed) edges of the patch (``neighborlist_changes``), the changed particles
    keeping their system, inclusion and exclusion labels."""
    from .neighborlist import neighborlist_changes

    idx = _i32(patch.indices).long()
    sysi = _i32(system)
    incl = _i32(inclusion) if inclusion is not None else sysi
    excl = _i32(exclusion) if exclusion is not None else torch.arange(sysi.shape[0], device="cuda",
                                                                      dtype=torch.int32)
    lh = NeighborListPoints(_f64(positions), sysi, incl, excl)
    rh = NeighborListPoints(_f64(patch.positions), sysi[idx], incl[idx], excl[idx])
    return neighborlist_changes(neighborlist, lh, patch.indices, rh, tril, cutoffs)


@dataclass
class LennardJonesParameters:
    labels: tuple
    sigma: torch.Tensor  # [T, T]
    epsilon: torch.Tensor  # [T, T]
    cutoff: torch.Tensor  # [S]

    @classmethod
    def from_lorentz_berthelot_mixing(cls, labels, sigma, epsilon, cutoff) -> "LennardJonesParameters":
        """sigma_ij = (sigma_i + sigma_j) / 2, eps_ij = sqrt(eps_i eps_j) (lennard_jones.py:125-141)."""
        s = torch.as_tensor(sigma, dtype=torch.float64)
        e = torch.as_tensor(epsilon, dtype=torch.float64)
        return cls(tuple(labels), (s[:, None] + s) / 2, torch.sqrt(e[:, None] * e),
                   torch.as_tensor(cutoff, dtype=torch.float64).reshape(-1))

    @classmethod
    def from_dict(cls, cutoff, parameters: dict, mixing_rule: str = "lorentz_berthelot"):
        """Missing sigma defaults to 1.0 and epsilon to 0.0 (lennard_jones.py:98-123)."""
        if mixing_rule != "lorentz_berthelot":
            raise ValueError(f"unknown mixing rule {mixing_rule}")
        labels = tuple(parameters.keys())
        raw = [(s or 1.0, e or 0.0) for s, e in parameters.values()]
        return cls.from_lorentz_berthelot_mixing(labels, [r[0] for r in raw], [r[1] for r in raw], [cutoff])


@dataclass
class LJParticles:
    positions: torch.Tensor  # f64 [N, 3]
    species: torch.Tensor  # int [N] index into the parameter tables
    system: torch.Tensor  # int [N]
    inclusion: torch.Tensor | None = None
    exclusion: torch.Tensor | None = None


@dataclass
class LJState:
    particles: LJParticles
    systems: Any  # tril [S, 6] or an object with .unitcell
    parameters: LennardJonesParameters


class LennardJonesPotential:
    """``Potential.__call__(state, patch=None) -> PotentialOut`` on the GPU."""

    def __init__(self, neighborlist: CellListNeighborList | None = None, pair_fp32: bool = True):
        self.neighborlist = neighborlist or CellListNeighborList()
        self.pair_fp32 = pair_fp32

    def __call__(self, state: LJState, patch: ParticlePatch | None = None, cache=None) -> PotentialOut:
        """Energies and gradients of ``state``; with ``patch``, the energies of ``state`` after the
        patch, E_cached - E(removed edges, old positions) + E(added edges, new positions)
        (``LocalGraphSumComposer``, src/kups/potential/common/graph.py:419-453, over the edges of
        ``neighborlist_changes``), no gradients.  ``cache`` is the ``cache`` of the
        PotentialOut of ``state`` (computed here when not given)."""
        p = state.particles
        tril = _f64(as_tril(state.systems))
        s = tril.shape[0]
        prm = state.parameters
        cut = _f64(prm.cutoff.reshape(-1).expand(s))
        if patch is not None:
            e_old = cache if cache is not None else self(state).cache
            added, removed = changed_edges(self.neighborlist, p.positions, p.system, p.inclusion, p.exclusion, tril,
                                           cut, patch)
            new_pos = patched_positions(p.positions, patch)
            e_rm = lj_from_edges(p.positions, p.system, p.species, tril, prm.sigma, prm.epsilon, cut, removed.indices,
                                 removed.shifts, removed.n_edges, self.pair_fp32).total_energies
            e_add = lj_from_edges(new_pos, p.system, p.species, tril, prm.sigma, prm.epsilon, cut, added.indices,
                                  added.shifts, added.n_edges, self.pair_fp32).total_energies
            e_new = e_old - e_rm + e_add
            return PotentialOut(e_new, None, None, cache=e_new)
        pts = NeighborListPoints(p.positions, p.system, p.inclusion, p.exclusion)
        edges, self.neighborlist = self.neighborlist.call_and_fix(pts, None, tril, cut)
        out = lj_from_edges(p.positions, p.system, p.species, tril, prm.sigma, prm.epsilon, cut, edges.indices,
                            edges.shifts, edges.n_edges, self.pair_fp32)
        out.cache = out.total_energies
        return out


def lj_from_edges(positions, system, species, tril, sigma, epsilon, cutoffs, edges, shifts, n_edges,
                  pair_fp32: bool = True) -> PotentialOut:
    lib = _lib.load()
    pos = _f64(positions)
    n = pos.shape[0]
    sysi = _i32(system)
    sp = _i32(species)
    tril = _f64(tril)
    s = tril.shape[0]
    cut = _f64(torch.as_tensor(cutoffs).reshape(-1).expand(s))
    sig = _f64(torch.as_tensor(sigma))
    eps = _f64(torch.as_tensor(epsilon))
    t = sig.shape[0]
    e_idx = _i32(edges).reshape(-1, 2)
    e_sh = _i32(shifts).reshape(-1, 3)
    energy = torch.empty(s, device="cuda", dtype=torch.float64)
    grad = torch.empty((n, 3), device="cuda", dtype=torch.float64)
    gtril = torch.empty((s, 6), device="cuda", dtype=torch.float64)
    status = new_status()
    rc = lib.kups_lj_edges(pos.data_ptr(), sysi.data_ptr(), sp.data_ptr(), n, tril.data_ptr(), cut.data_ptr(), s,
                           sig.data_ptr(), eps.data_ptr(), t, e_idx.data_ptr(), e_sh.data_ptr(), int(n_edges),
                           energy.data_ptr(), grad.data_ptr(), gtril.data_ptr(), int(bool(pair_fp32)),
                           status.data_ptr(), _stream())
    _lib.check(rc, "kups_lj_edges")
    _lib.raise_status(read_status(status))
    return PotentialOut(energy, PositionAndUnitCell(grad, gtril))


def make_lennard_jones_potential(neighborlist=None, pair_fp32: bool = True) -> LennardJonesPotential:
    return LennardJonesPotential(neighborlist, pair_fp32)


def lennard_jones_tail_correction(species, system, tril, sigma, epsilon, cutoffs, tail_mask=None, status=None):
    """Global analytic tail energy and pressure per system (lennard_jones.py:276-340).

    Atoms must be grouped by system.  ``tail_mask`` [T, T] selects the corrected species pairs
    (default: pairs with epsilon > 0).  Returns (energy [S], pressure [S]), float64.
    """
    from .neighborlist import _f64, _i32, _stream, new_status, read_status

    t = lambda x: torch.as_tensor(x)
    sp = _i32(t(species))
    sysi = _i32(t(system))
    tr = _f64(t(tril)).reshape(-1, 6).contiguous()
    s = tr.shape[0]
    sig, eps = _f64(t(sigma)), _f64(t(epsilon))
    nsp = int(sig.shape[0])
    rc = _f64(torch.as_tensor(cutoffs, dtype=torch.float64).reshape(-1).expand(s).contiguous())
    off = torch.zeros(s + 1, dtype=torch.int32, device="cuda")
    off[1:] = torch.cumsum(torch.bincount(sysi.to(torch.int64), minlength=s), 0).to(torch.int32)
    mask = _i32(t(tail_mask).to(torch.int32)) if tail_mask is not None else None
    e = torch.empty(s, dtype=torch.float64, device="cuda")
    p = torch.empty(s, dtype=torch.float64, device="cuda")
    st = status if status is not None else new_status()
    rcode = _lib.load().kups_lj_tail_correction(sp.data_ptr(), off.data_ptr(), s, tr.data_ptr(), sig.data_ptr(),
                                                eps.data_ptr(), mask.data_ptr() if mask is not None else None, nsp,
                                                rc.data_ptr(), e.data_ptr(), p.data_ptr(), st.data_ptr(), _stream())
    _lib.check(rcode, "kups_lj_tail_correction")
    if status is None:
        _lib.raise_status(read_status(st))
    return e, p
