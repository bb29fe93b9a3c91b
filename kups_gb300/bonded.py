"""Bonded edge-set potentials (bonds, angles, dihedrals, inversions) on the GPU.

Mirrors the parameter classes and energies of src/kups/potential/classical/
(``HarmonicBondParameters`` / ``harmonic_bond_energy`` and ``HarmonicAngleParameters`` /
``harmonic_angle_energy``, harmonic.py:64-163; ``MorseBondParameters``, morse.py:71-171;
``CosineAngleParameters``, cosine_angle.py:76-221; ``DihedralParameters``,
dihedral.py:73-273; ``InversionParameters``, inversion.py:86-209) as evaluated on the
HyperGraph of an ``EdgeSetGraphConstructor`` (potential/common/graph.py:289-361): a
fixed edge set of order 2, 3 or 4 with integer image shifts, species-indexed parameter
tensors, and the gradients the reference takes by ``jax.vjp`` with respect to positions
and unit cell.  One call of ``kups_bonded_edges`` per term; several terms add into one
set of energy / gradient buffers (``evaluate``).
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status


def _t(x):
    return torch.as_tensor(np.asarray(x, np.float64), dtype=torch.float64)


@dataclass
class HarmonicBondParameters:
    labels: tuple
    x0: np.ndarray  # [T, T] A
    k: np.ndarray  # [T, T] energy / A^2
    kind = 0

    def table(self):
        return np.stack([np.asarray(self.x0, np.float64), np.asarray(self.k, np.float64)], -1)


@dataclass
class MorseBondParameters:
    labels: tuple
    r0: np.ndarray  # [T, T]
    D: np.ndarray
    alpha: np.ndarray
    kind = 1

    @classmethod
    def from_harmonic(cls, labels, r0, k, D):
        """alpha = sqrt(k / D) (morse.py:86-102)."""
        return cls(tuple(labels), np.asarray(r0), np.asarray(D), np.sqrt(np.asarray(k) / np.asarray(D)))

    def table(self):
        return np.stack([np.asarray(a, np.float64) for a in (self.r0, self.D, self.alpha)], -1)


@dataclass
class HarmonicAngleParameters:
    labels: tuple
    theta0: np.ndarray  # [T, T, T] degrees
    k: np.ndarray  # [T, T, T] energy / degree^2
    kind = 2

    def table(self):
        return np.stack([np.asarray(self.theta0, np.float64), np.asarray(self.k, np.float64)], -1)


@dataclass
class CosineAngleParameters:
    labels: tuple
    theta0: np.ndarray  # [T, T, T] radians
    k: np.ndarray  # [T, T, T] energy
    linear_tol: float = math.radians(5)
    kind = 3

    def table(self):
        t = np.asarray(self.theta0, np.float64)
        return np.stack([t, np.asarray(self.k, np.float64), np.full(t.shape, float(self.linear_tol))], -1)


@dataclass
class DihedralParameters:
    labels: tuple
    V: np.ndarray  # [T, T, T, T] energy
    n: np.ndarray  # periodicity
    phi0: np.ndarray  # radians
    kind = 4

    def table(self):
        return np.stack([np.asarray(a, np.float64) for a in (self.V, self.n, self.phi0)], -1)


@dataclass
class InversionParameters:
    labels: tuple
    omega0: np.ndarray  # [T, T, T, T] radians (atom 0 the centre)
    k: np.ndarray  # energy
    kind = 5

    def table(self):
        return np.stack([np.asarray(self.omega0, np.float64), np.asarray(self.k, np.float64)], -1)


@dataclass
class BondedTerm:
    """One bonded potential over a fixed edge set (the reference's EdgeSetGraphConstructor):
    edges [E, order] particle indices, shifts [E, order - 1, 3] integer image shifts of
    atoms 1.. relative to atom 0."""

    parameters: object
    edges: np.ndarray
    shifts: np.ndarray | None = None
    fp32: bool = False  # per-edge arithmetic in float32 (sums and differences stay float64)

    def __post_init__(self):
        lib = _lib.load()
        kind = self.parameters.kind
        self.order = lib.kups_bonded_order(kind)
        e = np.asarray(self.edges, np.int32).reshape(-1, self.order)
        sh = (np.zeros((len(e), self.order - 1, 3), np.int32) if self.shifts is None
              else np.asarray(self.shifts, np.int32).reshape(len(e), self.order - 1, 3))
        tab = self.parameters.table()
        self.n_species = tab.shape[0]
        if tab.shape != (self.n_species,) * self.order + (lib.kups_bonded_param_count(kind),):
            raise ValueError(f"parameter tensors of {type(self.parameters).__name__} must be "
                             f"[T]*{self.order} (got {tab.shape[:-1]})")
        self._edges = torch.as_tensor(e).cuda().contiguous()
        self._shifts = torch.as_tensor(sh).cuda().contiguous()
        self._table = torch.as_tensor(tab.reshape(-1)).cuda().contiguous()

    def add_to(self, positions, system, species, tril, energy, grad, grad_tril, status):
        rc = _lib.load().kups_bonded_edges(
            self.parameters.kind, positions.data_ptr(), system.data_ptr(), species.data_ptr(), positions.shape[0],
            tril.data_ptr(), tril.shape[0], self._edges.data_ptr(), self._shifts.data_ptr(), self._edges.shape[0],
            self._table.data_ptr(), self.n_species, energy.data_ptr(), grad.data_ptr(),
            grad_tril.data_ptr() if grad_tril is not None else None, int(self.fp32), status.data_ptr(), _stream())
        _lib.check(rc, "kups_bonded_edges")

    def incidence(self, n_particles):
        """Atom -> edge lists (CSR: offsets int64 [n + 1], edge ids int32), each (atom, edge)
        pair once; built on the device once per particle count (the edge set is fixed)."""
        cache = getattr(self, "_incidence", None)
        if cache is not None and cache[0] == n_particles:
            return cache[1], cache[2]
        E = self._edges.shape[0]
        atoms = self._edges.reshape(-1).to(torch.int64)
        eid = torch.arange(E, device="cuda", dtype=torch.int64).repeat_interleave(self.order)
        ok = (atoms >= 0) & (atoms < n_particles)
        key = torch.unique(atoms[ok] * max(E, 1) + eid[ok])
        atom = key // max(E, 1)
        offsets = torch.zeros(n_particles + 1, dtype=torch.int64, device="cuda")
        offsets[1:] = torch.cumsum(torch.bincount(atom, minlength=n_particles), 0)
        edges = (key % max(E, 1)).to(torch.int32).contiguous()
        self._incidence = (n_particles, offsets, edges)
        return offsets, edges

    def add_delta(self, positions, system, species, tril, changed, new_positions, new_image, delta, workspace, status,
                  use_incidence=True):
        """delta[s] += E(new) - E(old) over this term's edges that touch a changed particle
        (through the incidence lists, or by scanning every edge)."""
        ws_bytes = workspace.numel()
        off, inc = self.incidence(positions.shape[0]) if use_incidence else (None, None)
        rc = _lib.load().kups_bonded_delta(
            self.parameters.kind, positions.data_ptr(), system.data_ptr(), species.data_ptr(), positions.shape[0],
            tril.data_ptr(), tril.shape[0], self._edges.data_ptr(), self._shifts.data_ptr(), self._edges.shape[0],
            self._table.data_ptr(), self.n_species, off.data_ptr() if off is not None else None,
            inc.data_ptr() if inc is not None else None, changed.data_ptr(), new_positions.data_ptr(),
            new_image.data_ptr() if new_image is not None else None, changed.shape[0], delta.data_ptr(),
            int(self.fp32), workspace.data_ptr(), ws_bytes, status.data_ptr(), _stream())
        _lib.check(rc, "kups_bonded_delta")


def evaluate(terms, positions, system, species, tril):
    """Sum of bonded terms: (energy [S], dE/dx [N, 3], dE/dtril [S, 6]), float64 device tensors."""
    dev = "cuda"
    pos = torch.as_tensor(positions, dtype=torch.float64, device=dev).contiguous()
    sysi = torch.as_tensor(system, device=dev).to(torch.int32).contiguous()
    spc = torch.as_tensor(species, device=dev).to(torch.int32).contiguous()
    tr = torch.as_tensor(tril, dtype=torch.float64, device=dev).contiguous()
    S = tr.shape[0]
    energy = torch.zeros(S, dtype=torch.float64, device=dev)
    grad = torch.zeros_like(pos)
    grad_tril = torch.zeros((S, 6), dtype=torch.float64, device=dev)
    status = new_status()
    for t in terms:
        t.add_to(pos, sysi, spc, tr, energy, grad, grad_tril, status)
    _lib.raise_status(read_status(status))
    return energy, grad, grad_tril


def delta_energy(terms, positions, system, species, tril, changed, new_positions, new_image=None, use_incidence=True):
    """MC energy change [S] of a sum of bonded terms when the particles `changed` move to
    `new_positions` (the old-graph / new-graph difference of the reference's
    LocalGraphSumComposer, potential/common/graph.py:412-450); ``new_image`` [k, 3] gives the
    lattice offset n of each moved atom whose new position was wrapped (new = unwrapped - n @ L)."""
    dev = "cuda"
    pos = torch.as_tensor(positions, dtype=torch.float64, device=dev).contiguous()
    sysi = torch.as_tensor(system, device=dev).to(torch.int32).contiguous()
    spc = torch.as_tensor(species, device=dev).to(torch.int32).contiguous()
    tr = torch.as_tensor(tril, dtype=torch.float64, device=dev).contiguous()
    ch = torch.as_tensor(changed, device=dev).to(torch.int32).contiguous()
    npos = torch.as_tensor(new_positions, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    img = (torch.as_tensor(new_image, device=dev).to(torch.int32).reshape(-1, 3).contiguous()
           if new_image is not None else None)
    delta = torch.zeros(tr.shape[0], dtype=torch.float64, device=dev)
    ws = torch.empty(_lib.load().kups_bonded_delta_workspace_bytes(pos.shape[0]), dtype=torch.uint8, device=dev)
    status = new_status()
    for t in terms:
        t.add_delta(pos, sysi, spc, tr, ch, npos, img, delta, ws, status, use_incidence)
    _lib.raise_status(read_status(status))
    return delta
