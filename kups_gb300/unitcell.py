"""Lower-triangular unit cells (host side).

Mirrors ``TriclinicUnitCell`` (src/kups/core/unitcell.py:251-380): ``tril`` =
[L00, L10, L11, L20, L21, L22] per system, row convention r = f @ L.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import torch

TRIL_IDX = ((0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2))


@dataclass
class TriclinicUnitCell:
    tril: torch.Tensor  # [S, 6]

    @classmethod
    def from_matrix(cls, vecs) -> "TriclinicUnitCell":
        v = torch.as_tensor(vecs, dtype=torch.float64)
        return cls(torch.stack([v[..., a, b] for a, b in TRIL_IDX], -1))

    @classmethod
    def from_lengths_and_angles(cls, lengths, angles) -> "TriclinicUnitCell":
        """unitcell.py:99-136."""
        a, b, c = (float(x) for x in lengths)
        al, be, ga = (math.radians(float(x)) for x in angles)
        ca, cb, cg, sg = math.cos(al), math.cos(be), math.cos(ga), math.sin(ga)
        c2z = c * math.sqrt(1 - ca**2 - cb**2 - cg**2 + 2 * ca * cb * cg) / sg
        m = [[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [c * cb, c * (ca - cb * cg) / sg, c2z]]
        return cls.from_matrix(torch.tensor(m, dtype=torch.float64)[None])

    @property
    def lattice_vectors(self) -> torch.Tensor:
        L = torch.zeros(self.tril.shape[:-1] + (3, 3), dtype=self.tril.dtype, device=self.tril.device)
        for k, (a, b) in enumerate(TRIL_IDX):
            L[..., a, b] = self.tril[..., k]
        return L

    @property
    def volume(self) -> torch.Tensor:
        t = self.tril
        return (t[..., 0] * t[..., 2] * t[..., 5]).abs()


def as_tril(systems) -> torch.Tensor:
    """Accept a tensor [S, 6], a TriclinicUnitCell, or an object with .unitcell / .tril."""
    if isinstance(systems, torch.Tensor):
        return systems
    if isinstance(systems, TriclinicUnitCell):
        return systems.tril
    if hasattr(systems, "unitcell"):
        return as_tril(systems.unitcell)
    if hasattr(systems, "tril"):
        return systems.tril
    return torch.as_tensor(systems, dtype=torch.float64)
