"""Per-system virial observables in float64 (oracle, test infrastructure).

Restates src/kups/observables/stress.py: the atomic virial stress
(``_stress_via_virial_theorem``, :70-82, through ``oracle.md.virial_stress``), the
molecular virial stress of the RASPA convention (``_molecular_stress_via_virial_theorem``,
:85-118), the lattice-gradient stress (:64-67); src/kups/observables/pressure.py
(``_pressure_from_stress`` :27-29, ``_ideal_gas_pressure`` :32-36) and
src/kups/md/observables.py (``particle_kinetic_energy`` :17-35, ``instantaneous_pressure``
:38-61).  One deliberate difference: the reference divides the molecular stress of every
system by the volume of the first system (``system_volume[:1]``, stress.py:114); here each
system uses its own volume, which is the same number for one system or equal cells.
"""

from __future__ import annotations

import numpy as np

from .md import instantaneous_pressure, kinetic_energy, virial_stress
from .unitcell import lattice_from_tril, volume, wrap
from .units import BOLTZMANN_CONSTANT

__all__ = ["virial_stress", "molecular_virial_stress", "lattice_stress", "pressure_from_stress",
           "ideal_gas_pressure", "instantaneous_pressure", "kinetic_energy", "group_centres"]


def group_centres(pos, group, n_groups, system, tril):
    """Centre of each group: the atoms' minimum images relative to the group's first atom,
    averaged, shifted back by that atom and wrapped into the primary cell [-0.5, 0.5)
    (stress.py:96-108; the reference's anchor is whichever atom its scatter keeps, which
    gives the same centre for molecules smaller than half the cell)."""
    pos = np.asarray(pos, np.float64)
    group = np.asarray(group)
    sysi = np.asarray(system)
    tril = np.asarray(tril, np.float64)
    first = np.full(n_groups, len(pos), np.int64)
    np.minimum.at(first, group, np.arange(len(pos)))
    has = first < len(pos)
    anchor = np.where(has, first, 0)
    offsets = pos[anchor]
    rel = wrap(pos - offsets[group], tril[sysi])
    com = np.zeros((n_groups, 3))
    np.add.at(com, group, rel)
    counts = np.bincount(group, minlength=n_groups)[:, None]
    gsys = np.zeros(n_groups, np.int64)
    gsys[group] = sysi
    com = com / np.maximum(counts, 1) + offsets
    return wrap(com, tril[gsys]), has


def molecular_virial_stress(pos, grad, system, group, n_groups, tril, dtril):
    """sigma = -(sym(sum_i (r_i - wrap(r_i - R_g(i))) (x) dU/dr_i) + h^T dU/dh) / V, sym(A) =
    (A + A^T) / 2, R_g the wrapped centre of the atom's group (stress.py:85-118)."""
    pos = np.asarray(pos, np.float64)
    sysi = np.asarray(system)
    group = np.asarray(group)
    tril = np.asarray(tril, np.float64)
    com, _ = group_centres(pos, group, n_groups, sysi, tril)
    rel_pos = wrap(pos - com[group], tril[sysi])
    w = pos - rel_pos
    out = np.zeros((tril.shape[0], 3, 3))
    np.add.at(out, sysi, w[:, :, None] * np.asarray(grad, np.float64)[:, None, :])
    out = -out
    out = 0.5 * (out + np.swapaxes(out, 1, 2))
    for s in range(tril.shape[0]):
        L = lattice_from_tril(tril[s])
        G = lattice_from_tril(np.asarray(dtril)[s])
        out[s] = (out[s] - L.T @ G) / volume(tril[s])
    return out


def lattice_stress(tril, dtril):
    """sigma = -dU/dh / V (stress.py:64-67)."""
    return -lattice_from_tril(np.asarray(dtril, np.float64)) / volume(tril)[:, None, None]


def pressure_from_stress(stress):
    """P = Tr(sigma) / 3 (pressure.py:27-29)."""
    return np.trace(np.asarray(stress), axis1=-2, axis2=-1) / 3


def ideal_gas_pressure(counts, temperature, tril):
    """P = N k_B T / V (pressure.py:32-36)."""
    return np.asarray(counts, np.float64) * BOLTZMANN_CONSTANT * np.asarray(temperature, np.float64) / volume(tril)
