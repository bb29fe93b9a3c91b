"""Bonded edge-set potentials in float64 (oracle, test infrastructure).

Restates, per edge of order D with atoms (i_0, ..., i_{D-1}) and integer image shifts
s_1..s_{D-1}, the difference vectors v_m = x_{i_m} - x_{i_0} + s_m @ L
(``Edges.difference_vectors``, src/kups/core/neighborlist.py:164-204) and the energies of
src/kups/potential/classical/:
  harmonic bond   k (|v1| - x0)^2                                  (harmonic.py:83-108)
  Morse bond      D (1 - exp(-alpha (|v1| - r0)))^2                (morse.py:142-171)
  harmonic angle  k (theta_deg - theta0_deg)^2, theta at atom 0    (harmonic.py:130-163)
  cosine angle    K (1 + cos t) near linear, else K (C0 + C1 cos t + C2 cos 2t)
                                                                   (cosine_angle.py:152-221)
  dihedral        V / 2 (1 - cos(n phi0) cos(n phi)), atan2 form   (dihedral.py:214-273)
  inversion       k_s (C0 + C1 cos w + C2 cos 2w), w out of plane  (inversion.py:136-209)
with the reference's 1e-10 regularisers.  Energies are summed per system (over the first
atom's system); gradients dE/dx and dE/dtril (Cartesian positions fixed) come from central
differences of the per-edge energies with respect to the difference vectors, an
evaluation independent of the kernel's analytic derivatives.
"""

from __future__ import annotations

import numpy as np

from .unitcell import lattice_from_tril

KINDS = {"harmonic_bond": (0, 2), "morse_bond": (1, 2), "harmonic_angle": (2, 3), "cosine_angle": (3, 3),
         "dihedral": (4, 4), "inversion": (5, 4)}
EPS = 1e-10


def difference_vectors(pos, system, tril, edges, shifts):
    pos = np.asarray(pos, np.float64)
    edges = np.asarray(edges)
    L = lattice_from_tril(np.asarray(tril, np.float64))[np.asarray(system)[edges[:, 0]]]  # [E, 3, 3]
    sh = np.asarray(shifts, np.float64).reshape(len(edges), edges.shape[1] - 1, 3)
    return pos[edges[:, 1:]] - pos[edges[:, :1]] + np.einsum("emk,ekl->eml", sh, L)


def cosine_coefficients(theta0):
    sin2 = np.sin(theta0) ** 2
    c = np.cos(theta0)
    c2 = 1.0 / (4.0 * np.maximum(sin2, 1e-10))
    return c2 * (2.0 * c**2 + 1.0), -4.0 * c2 * c, c2


def edge_energy(kind: str, v, p):
    """Per-edge energies; v [E, D-1, 3], p [E, n_params] (the parameter table rows)."""
    if kind in ("harmonic_bond", "morse_bond"):
        r = np.linalg.norm(v[:, 0], axis=-1)
        if kind == "harmonic_bond":
            return (r - p[:, 0]) ** 2 * p[:, 1]
        return p[:, 1] * (1 - np.exp(-p[:, 2] * (r - p[:, 0]))) ** 2
    if kind in ("harmonic_angle", "cosine_angle"):
        v1, v2 = v[:, 0], v[:, 1]
        c = np.einsum("ij,ij->i", v1, v2) / (np.linalg.norm(v1, axis=-1) * np.linalg.norm(v2, axis=-1))
        if kind == "harmonic_angle":
            return (np.rad2deg(np.arccos(c)) - p[:, 0]) ** 2 * p[:, 1]
        c = np.clip(c, -1.0, 1.0)
        theta0, k, tol = p[:, 0], p[:, 1], p[:, 2]
        c0, c1, c2 = cosine_coefficients(theta0)
        general = k * (c0 + c1 * c + c2 * (2.0 * c**2 - 1.0))
        return np.where(np.abs(theta0 - np.pi) < tol, k * (1.0 + c), general)
    if kind == "dihedral":
        r_ij = v[:, 0]
        r_jk = v[:, 1] - r_ij
        r_kl = v[:, 2] - v[:, 1]
        n1, n2 = np.cross(r_ij, r_jk), np.cross(r_jk, r_kl)
        n1 = n1 / (np.linalg.norm(n1, axis=-1, keepdims=True) + EPS)
        n2 = n2 / (np.linalg.norm(n2, axis=-1, keepdims=True) + EPS)
        cos_phi = np.sum(n1 * n2, axis=-1)
        b = r_jk / (np.linalg.norm(r_jk, axis=-1, keepdims=True) + EPS)
        sin_phi = np.sum(np.cross(n1, n2) * b, axis=-1)
        phi = np.arctan2(sin_phi, cos_phi)
        V, n, phi0 = p[:, 0], p[:, 1], p[:, 2]
        return 0.5 * V * (1.0 - np.cos(n * phi0) * np.cos(n * phi))
    if kind == "inversion":
        r_ji, r_jk, r_jl = v[:, 0], v[:, 1], v[:, 2]
        nv = np.cross(r_jk, r_jl)
        nv = nv / (np.linalg.norm(nv, axis=-1, keepdims=True) + EPS)
        s = np.einsum("ij,ij->i", r_ji, nv) / (np.linalg.norm(r_ji, axis=-1) + EPS)
        w = np.arcsin(np.clip(s, -1.0, 1.0))
        omega0, k = p[:, 0], p[:, 1]
        sin2, cw0 = np.sin(omega0) ** 2, np.cos(omega0)
        sp2 = np.abs(omega0) < 1e-6
        c2 = np.where(sp2, 0.0, 1.0 / (4.0 * np.where(sin2 > 1e-10, sin2, 1.0)))
        c1 = np.where(sp2, -1.0, -4.0 * c2 * cw0)
        c0 = np.where(sp2, 1.0, c2 * (2.0 * cw0**2 + 1.0))
        ks = np.where(sp2, k, k / np.maximum(c0 + c1 + c2, 1e-10))
        return ks * (c0 + c1 * np.cos(w) + c2 * np.cos(2.0 * w))
    raise ValueError(kind)


def edge_parameters(table, species, edges, n_species):
    """Rows of the flattened [T^D, n_params] table for each edge's species tuple."""
    sp = np.asarray(species)[np.asarray(edges)]
    idx = np.zeros(len(sp), np.int64)
    for d in range(sp.shape[1]):
        idx = idx * n_species + sp[:, d]
    return np.asarray(table, np.float64)[idx]


def bonded(kind, pos, system, species, tril, table, n_species, edges, shifts, h=1e-6):
    """(energy [S], dE/dx [N, 3], dE/dtril [S, 6])."""
    edges = np.asarray(edges)
    tril = np.asarray(tril, np.float64)
    S, N = tril.shape[0], len(pos)
    v = difference_vectors(pos, system, tril, edges, shifts)
    p = edge_parameters(table, species, edges, n_species)
    sysi = np.asarray(system)[edges[:, 0]]
    e = edge_energy(kind, v, p)
    energy = np.zeros(S)
    np.add.at(energy, sysi, e)
    g = np.zeros_like(v)
    for m in range(v.shape[1]):
        for a in range(3):
            vp, vm = v.copy(), v.copy()
            vp[:, m, a] += h
            vm[:, m, a] -= h
            g[:, m, a] = (edge_energy(kind, vp, p) - edge_energy(kind, vm, p)) / (2 * h)
    grad = np.zeros((N, 3))
    for m in range(v.shape[1]):
        np.add.at(grad, edges[:, m + 1], g[:, m])
        np.add.at(grad, edges[:, 0], -g[:, m])
    sh = np.asarray(shifts, np.float64).reshape(len(edges), v.shape[1], 3)
    dl = np.einsum("ema,emb->eab", sh, g)  # dE/dL_ab = sum_m s_ma g_mb
    gt = np.zeros((S, 6))
    for k, (a, b) in enumerate(((0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2))):
        np.add.at(gt[:, k], sysi, dl[:, a, b])
    return energy, grad, gt
