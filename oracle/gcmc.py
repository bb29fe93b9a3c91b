"""Total energy of a GCMC configuration in float64 (oracle, test infrastructure).

Restates the potential that src/kups/application/simulations/mcmc_rigid.py:281-307
sums for rigid-molecule GCMC: Lennard-Jones over the reference neighbour list
(lennard_jones.py:149-178), Ewald short range with exclusion = molecule
(ewald.py:305-325, exclusion on the minimum image only, neighborlist.py:731-735),
long range (:585-601), self (:277-302), the intramolecular exclusion correction
(:328-346) and the global LJ tail correction (lennard_jones.py:276-315).
Energy differences of two configurations are what the GPU MC step computes
incrementally.  Framework atoms share one exclusion label (a rigid host; its
internal terms cancel in every difference).
"""

from __future__ import annotations

import numpy as np

from . import ewald, lennard_jones, neighborlist


def total_energy(fw_pos, fw_species, fw_q, guests, motif_species, motif_q, tril, sigma, epsilon, rc_lj, rc_ew,
                 alpha, kvec_n, tail=True):
    """guests: [n_mol * apm, 3]; one system; returns the total energy (eV)."""
    apm = len(motif_q)
    guests = np.asarray(guests, float).reshape(-1, 3)
    m = len(guests) // apm
    pos = np.concatenate([fw_pos, guests])
    sp = np.concatenate([fw_species, np.tile(motif_species, m)])
    q = np.concatenate([fw_q, np.tile(motif_q, m)])
    n_fw = len(fw_pos)
    excl = np.concatenate([np.full(n_fw, -1), np.repeat(np.arange(m), apm)])
    sysi = np.zeros(len(pos), int)
    tril = np.asarray(tril, float).reshape(1, 6)
    e_lj, s_lj = neighborlist.neighbor_list(pos, sysi, tril, [rc_lj], exclusion=excl)
    e_ew, s_ew = neighborlist.neighbor_list(pos, sysi, tril, [rc_ew], exclusion=excl)
    E = lennard_jones.lj_from_edges(pos, sysi, sp, tril, sigma, epsilon, [rc_lj], e_lj, s_lj)[0][0]
    E += ewald.short_range_from_edges(pos, q, sysi, tril, alpha, [rc_ew], e_ew, s_ew)[0][0]
    E += ewald.long_range(pos, q, sysi, tril, np.asarray(kvec_n)[None], alpha)[0][0]
    E += ewald.self_energy(q, sysi, alpha, 1)[0]
    # intramolecular pairs of the guests (minimum image), both directions
    xe = []
    for g in range(m):
        for a in range(apm):
            for b in range(apm):
                if a != b:
                    xe.append((n_fw + g * apm + a, n_fw + g * apm + b))
    if xe:
        xe = np.array(xe)
        from .unitcell import to_fractional

        f = to_fractional(pos, tril[0])
        xs = np.round(f[xe[:, 0]] - f[xe[:, 1]]).astype(np.int64)
        E += ewald.short_range_from_edges(pos, q, sysi, tril, alpha, [np.inf], xe, xs)[0][0]
        E -= ewald.coulomb_vacuum_from_edges(pos, q, sysi, tril, xe, xs, 1)[0]
    if tail:
        counts = np.bincount(sp, minlength=np.asarray(sigma).shape[0])[None].astype(float)
        mask = np.asarray(epsilon) > 0
        E += lennard_jones.tail_correction_energy(counts, tril, sigma, epsilon, [rc_lj], mask)[0]
    return float(E)
