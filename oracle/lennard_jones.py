"""Lennard-Jones energy, forces and cell gradient in float64 (oracle, test infrastructure).

Restates src/kups/potential/classical/lennard_jones.py:
``from_lorentz_berthelot_mixing`` (:125-141), ``lennard_jones_edge_energy``
(:149-168: 4 eps (c6^2 - c6) [r^2 < rc^2], c6 = (sigma^2/r^2)^3, truncated,
not shifted), ``lennard_jones_energy`` (:171-178: per-system edge sum / 2) and
the global tail correction (:276-315).  The reference obtains gradients by
``jax.vjp`` with respect to ``PositionAndUnitCell`` (potential/common/energy.py:264-355,
lennard_jones.py:481-488): positions are held fixed in Cartesian space while the
cell's ``tril`` varies through the edge shift term s @ L.  The analytic form
used here is dE/dx and dE/dL_ab = sum_edges 1/2 s_a g_b, g = dE_edge/dd.
"""

from __future__ import annotations

import numpy as np

from .neighborlist import difference_vectors
from .unitcell import TRIL_IDX, volume


def lorentz_berthelot(sigma, epsilon):
    sigma = np.asarray(sigma, dtype=np.float64)
    epsilon = np.asarray(epsilon, dtype=np.float64)
    return (sigma[:, None] + sigma) / 2, np.sqrt(epsilon[:, None] * epsilon)


def edge_terms(d, sig, eps, rc):
    """Per-edge energy and dE/dd for difference vectors d (directed edges)."""
    r2 = np.sum(d * d, axis=-1)
    c6 = (sig**2 / r2) ** 3
    mask = r2 < rc**2
    e = np.where(mask, 4 * eps * (c6**2 - c6), 0.0)
    # dE/dr2 = 4 eps (2 c6 - 1) dc6/dr2, dc6/dr2 = -3 c6 / r2
    dedr2 = np.where(mask, -12.0 * eps * c6 * (2 * c6 - 1) / r2, 0.0)
    g = 2.0 * dedr2[:, None] * d
    return e, g


def lj_from_edges(positions, system, species, tril, sigma, epsilon, cutoffs, edges, shifts):
    """Energy [S], dE/dx [N,3], dE/dtril [S,6] from a directed edge list."""
    pos = np.asarray(positions, dtype=np.float64)
    system = np.asarray(system, dtype=np.int64)
    tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
    S = tril.shape[0]
    cut = np.broadcast_to(np.asarray(cutoffs, dtype=np.float64), (S,))
    edges = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    shifts = np.asarray(shifts, dtype=np.float64).reshape(-1, 3)
    energy = np.zeros(S)
    grad = np.zeros_like(pos)
    dtril = np.zeros((S, 6))
    if edges.shape[0] == 0:
        return energy, grad, dtril
    i, j = edges[:, 0], edges[:, 1]
    es = system[i]
    d = difference_vectors(pos, system, tril, edges, shifts)
    sp = np.asarray(species, dtype=np.int64)
    sig = np.asarray(sigma)[sp[i], sp[j]]
    eps = np.asarray(epsilon)[sp[i], sp[j]]
    e, g = edge_terms(d, sig, eps, cut[es])
    np.add.at(energy, es, 0.5 * e)
    np.add.at(grad, j, 0.5 * g)
    np.add.at(grad, i, -0.5 * g)
    for k, (a, b) in enumerate(TRIL_IDX):
        np.add.at(dtril[:, k], es, 0.5 * shifts[:, a] * g[:, b])
    return energy, grad, dtril


def tail_correction_energy(species_counts, tril, sigma, epsilon, cutoffs, tail_mask=None):
    """Global analytic tail energy per system (lennard_jones.py:276-315)."""
    counts = np.asarray(species_counts, dtype=np.float64)
    v = volume(np.asarray(tril, dtype=np.float64).reshape(-1, 6))[:, None, None]
    density = counts[:, :, None] * counts[:, None, :] / v
    sigma = np.asarray(sigma, dtype=np.float64)
    eps = np.asarray(epsilon, dtype=np.float64)
    rc = np.asarray(cutoffs, dtype=np.float64).reshape(-1)[:, None, None]
    t1 = (sigma / rc) ** 3
    t2 = t1**3
    res = (8 / 3) * np.pi * density * eps * sigma**3 * (t2 / 3 - t1)
    if tail_mask is None:
        tail_mask = eps > 0
    res = res * tail_mask
    return res.sum(axis=(1, 2))


def tail_correction_pressure(species_counts, tril, sigma, epsilon, cutoffs, tail_mask=None):
    """Global analytic tail pressure per system (lennard_jones.py:318-340)."""
    counts = np.asarray(species_counts, dtype=np.float64)
    v = volume(np.asarray(tril, dtype=np.float64).reshape(-1, 6))[:, None, None]
    density = counts[:, :, None] * counts[:, None, :] / v
    sigma = np.asarray(sigma, dtype=np.float64)
    eps = np.asarray(epsilon, dtype=np.float64)
    rc = np.asarray(cutoffs, dtype=np.float64).reshape(-1)[:, None, None]
    t1 = (sigma / rc) ** 3
    t2 = t1**3
    res = (16 / 3) * np.pi * density / v * eps * sigma**3 * (t2 / 3 * 2 - t1)
    if tail_mask is None:
        tail_mask = eps > 0
    res = res * tail_mask
    return res.sum(axis=(1, 2))
