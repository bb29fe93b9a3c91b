"""Ewald summation in float64 (oracle, test infrastructure).

Restates src/kups/potential/classical/ewald.py:
* ``TO_STANDARD_UNITS`` (:82), ``ewald_self_interaction_energy`` (:277-302),
  ``ewald_short_range_energy`` (:305-325), ``exclusion_correction_energy``
  (:328-346) with ``coulomb_vacuum_energy`` (coulomb.py:64-83);
* ``EwaldLongRangeInput.kvecs`` (:265-274: k = 2 pi L^-1 n), ``prefactor``
  (:363-391: (2 - [n_x = 0]) 2 pi / V exp(-k^2 / 4 alpha^2) / k^2, k = 0 masked),
  ``_frequency_response`` / ``_structure_factor_full`` (:394-439),
  ``long_range`` (:349-360), ``ewald_long_range_energy`` (:585-601);
* ``_structure_factor_update`` (:442-486) for incremental MC updates;
* ``estimate_ewald_parameters`` (:1166-1319) and ``kvecs_from_kmax`` (:1322-1339).

Gradients (the reference differentiates with ``jax.vjp``) are written out
analytically: dE/dr_i and dE/dtril with Cartesian positions held fixed.
"""

from __future__ import annotations

import numpy as np
from scipy import optimize, special

from .neighborlist import difference_vectors
from .unitcell import TRIL_IDX, inverse_tril, lattice_from_tril, perpendicular_lengths, volume
from .units import TO_STANDARD_UNITS as KE


# ----------------------------------------------------------------------------- k-vectors
def kvecs_from_kmax(tril: np.ndarray, kmax: float) -> np.ndarray:
    """Integer k coefficients n (half space n_x >= 0) with |2 pi L^-1 n| <= kmax."""
    inv = lattice_from_tril(inverse_tril(np.asarray(tril, dtype=np.float64)))
    rvecs = inv.T * 2 * np.pi
    min_length = np.min(np.linalg.svd(rvecs)[1])
    n = int(np.ceil(kmax / min_length))
    grids = np.meshgrid(np.arange(0, n + 1), np.arange(-n, n + 1), np.arange(-n, n + 1))
    vecs = np.stack(grids, axis=-1).reshape(-1, 3)
    k = vecs @ rvecs
    return vecs[np.linalg.norm(k, axis=-1) <= kmax].astype(np.int64)


def kvecs_cube(kmax_int: int) -> np.ndarray:
    """Half-space integer box |n|_inf <= kmax_int with n_x >= 0 (reference layout)."""
    m = int(kmax_int)
    grids = np.meshgrid(np.arange(0, m + 1), np.arange(-m, m + 1), np.arange(-m, m + 1))
    return np.stack(grids, axis=-1).reshape(-1, 3).astype(np.int64)


def cartesian_kvecs(tril_s: np.ndarray, n: np.ndarray) -> np.ndarray:
    inv = lattice_from_tril(inverse_tril(np.asarray(tril_s, dtype=np.float64)))
    return 2 * np.pi * np.asarray(n, dtype=np.float64) @ inv.T


def prefactor(tril_s, n, alpha):
    k = cartesian_kvecs(tril_s, n)
    k2 = np.sum(k * k, axis=-1)
    mask = k2 > 0
    k2s = np.where(mask, k2, 1.0)
    p = 2 * np.pi / volume(tril_s) * np.exp(-k2s / (4 * alpha**2)) / k2s
    p = (2 - (np.asarray(n)[:, 0] == 0)) * p
    return np.where(mask, p, 0.0), k, k2s, mask


# ----------------------------------------------------------------------------- energies
def self_energy(charges, system, alpha, n_systems):
    q2 = np.zeros(n_systems)
    np.add.at(q2, np.asarray(system), np.asarray(charges, dtype=np.float64) ** 2)
    return -q2 * np.asarray(alpha) / np.sqrt(np.pi) * KE


def structure_factor(positions, charges, system, tril, kvec_n):
    """S(k) [S, n_k, 2] with kvec_n int [S, n_k, 3] (zero rows are padding)."""
    S = tril.shape[0]
    out = np.zeros((S, kvec_n.shape[1], 2))
    for s in range(S):
        m = np.asarray(system) == s
        k = cartesian_kvecs(tril[s], kvec_n[s])
        th = np.asarray(positions)[m] @ k.T
        q = np.asarray(charges)[m][:, None]
        out[s, :, 0] = np.sum(q * np.cos(th), axis=0)
        out[s, :, 1] = np.sum(q * np.sin(th), axis=0)
    return out


def long_range(positions, charges, system, tril, kvec_n, alpha):
    """Reciprocal energy [S], dE/dx [N,3], dE/dtril [S,6], S(k)."""
    pos = np.asarray(positions, dtype=np.float64)
    q = np.asarray(charges, dtype=np.float64)
    system = np.asarray(system)
    tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
    S = tril.shape[0]
    alpha = np.broadcast_to(np.asarray(alpha, dtype=np.float64), (S,))
    energy = np.zeros(S)
    grad = np.zeros_like(pos)
    dtril = np.zeros((S, 6))
    sk_all = np.zeros((S, kvec_n.shape[1], 2))
    for s in range(S):
        m = np.nonzero(system == s)[0]
        P, k, k2, kmask = prefactor(tril[s], kvec_n[s], alpha[s])
        th = pos[m] @ k.T  # [n, nk]
        c, sn = np.cos(th), np.sin(th)
        Sc = q[m] @ c
        Ss = q[m] @ sn
        sk_all[s, :, 0], sk_all[s, :, 1] = Sc, Ss
        S2 = Sc * Sc + Ss * Ss
        e = KE * np.sum(P * S2)
        energy[s] = e
        # dE/dr_i = 2 K q_i sum_k P k (Ss cos - Sc sin)
        w = (Ss[None, :] * c - Sc[None, :] * sn) * P[None, :]  # [n, nk]
        grad[m] = 2 * KE * q[m][:, None] * (w @ k)
        # dE/dk = K [ |S|^2 dP/dk + P d|S|^2/dk ]
        dPdk = (P * (-1 / (2 * alpha[s] ** 2) - 2 / k2))[:, None] * k
        dS2dk = 2 * ((q[m][:, None] * (Ss[None, :] * c - Sc[None, :] * sn)).T @ pos[m])
        g = KE * (S2[:, None] * dPdk + P[:, None] * dS2dk)  # [nk, 3]
        inv = lattice_from_tril(inverse_tril(tril[s]))
        Lg = g @ inv  # rows: (L^-T g_k)^T = g_k^T L^-1
        dL = -(Lg.T @ k)  # [3, 3]: dE/dL_ab = -sum_k (L^-T g_k)_a k_b
        Ld = lattice_from_tril(tril[s])
        for a in range(3):
            dL[a, a] += -e / Ld[a, a]
        dtril[s] = [dL[a, b] for a, b in TRIL_IDX]
    return energy, grad, dtril, sk_all


def long_range_from_sk(sk, tril, kvec_n, alpha):
    S = tril.shape[0]
    out = np.zeros(S)
    for s in range(S):
        P = prefactor(tril[s], kvec_n[s], np.broadcast_to(alpha, (S,))[s])[0]
        out[s] = KE * np.sum(P * (sk[s, :, 0] ** 2 + sk[s, :, 1] ** 2))
    return out


def short_range_from_edges(positions, charges, system, tril, alpha, cutoffs, edges, shifts):
    """Real-space energy [S], dE/dx, dE/dtril over a directed edge list."""
    pos = np.asarray(positions, dtype=np.float64)
    q = np.asarray(charges, dtype=np.float64)
    system = np.asarray(system)
    tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
    S = tril.shape[0]
    alpha = np.broadcast_to(np.asarray(alpha, dtype=np.float64), (S,))
    cut = np.broadcast_to(np.asarray(cutoffs, dtype=np.float64), (S,))
    energy = np.zeros(S)
    grad = np.zeros_like(pos)
    dtril = np.zeros((S, 6))
    if len(edges) == 0:
        return energy, grad, dtril
    i, j = edges[:, 0], edges[:, 1]
    es = system[i]
    d = difference_vectors(pos, system, tril, edges, shifts)
    r = np.linalg.norm(d, axis=-1)
    a = alpha[es]
    qq = q[i] * q[j]
    mask = r < cut[es]
    erfc = special.erfc(a * r)
    e = np.where(mask, qq * erfc / r, 0.0)
    dedr = np.where(mask, qq * (-erfc / r**2 - 2 * a / np.sqrt(np.pi) * np.exp(-(a * r) ** 2) / r), 0.0)
    g = (dedr / r)[:, None] * d * KE
    np.add.at(energy, es, 0.5 * e * KE)
    np.add.at(grad, j, 0.5 * g)
    np.add.at(grad, i, -0.5 * g)
    sh = np.asarray(shifts, dtype=np.float64)
    for k, (aa, bb) in enumerate(TRIL_IDX):
        np.add.at(dtril[:, k], es, 0.5 * sh[:, aa] * g[:, bb])
    return energy, grad, dtril


def coulomb_vacuum_from_edges(positions, charges, system, tril, edges, shifts, n_systems):
    pos = np.asarray(positions, dtype=np.float64)
    q = np.asarray(charges, dtype=np.float64)
    energy = np.zeros(n_systems)
    if len(edges) == 0:
        return energy
    d = difference_vectors(pos, system, tril, edges, shifts)
    r = np.linalg.norm(d, axis=-1)
    np.add.at(energy, np.asarray(system)[edges[:, 0]], 0.5 * q[edges[:, 0]] * q[edges[:, 1]] / r * KE)
    return energy


# ----------------------------------------------------------------------------- parameters
def estimate_ewald_parameters(charges, tril, real_cutoff=None, alpha=None, epsilon_total=1e-8):
    """Grid-search parameter estimate (ewald.py:1166-1319). Returns dict."""
    q = np.asarray(charges, dtype=np.float64)
    tril = np.asarray(tril, dtype=np.float64).reshape(6)
    vol = float(volume(tril))
    Q2 = float(np.vdot(q, q))
    N = q.size
    max_radius = float(np.min(perpendicular_lengths(tril))) / 2
    eps_target = epsilon_total / 2
    lattice_length = vol ** (1 / 3)

    def minimize(f, bounds, n=200):
        attempts = np.linspace(bounds[0], bounds[1], n)
        return attempts[np.argmin([f(x) for x in attempts])]

    def real_err(rc, a):
        if rc <= 0 or a <= 0:
            return np.inf
        return (Q2 / np.sqrt(N)) * (special.erfc(a * rc) / rc)

    def recip_err(kc, a):
        if kc <= 0 or a <= 0:
            return np.inf
        x = -(kc**2) / (4 * a**2)
        if x < -700:
            return 0.0
        return (Q2 * a / (np.sqrt(N) * np.pi)) * np.exp(x)

    def opt_rc(a):
        if real_cutoff is None:
            rc = minimize(lambda rc: abs(real_err(rc, a) - eps_target), (0.01, min(20.0, max_radius)))
        else:
            rc = real_cutoff
        if real_err(rc, a) > eps_target * 2:
            return np.inf
        return rc

    def opt_kc(a):
        kc = minimize(lambda kc: abs(recip_err(kc, a) - eps_target), (0.1, 5.0))
        if recip_err(kc, a) > eps_target * 2:
            return np.inf
        return kc

    def cost(a):
        if a <= 0:
            return np.inf
        rc = opt_rc(a)
        if rc == np.inf:
            return np.inf
        kc = opt_kc(a)
        if kc == np.inf:
            return np.inf
        n_k = (2 * kc * lattice_length / 2 / np.pi + 1) ** 3
        return float(rc**3 * N / vol * 4 / 3 * np.pi + n_k)

    if real_cutoff is not None:
        target = real_cutoff * eps_target
        res = optimize.minimize_scalar(lambda z: abs(special.erfc(z) - target))
        if not res.success:
            raise ValueError("Failed to find alpha for given real space cutoff.")
        a = res.x / real_cutoff
        kmax = 2 * a * np.sqrt(-np.log(eps_target))
        return dict(alpha=a, real_cutoff=real_cutoff, k_max=kmax,
                    error_real=real_err(real_cutoff, a), error_recip=recip_err(kmax, a))
    a = minimize(cost, (0.001, 2), n=400) if alpha is None else alpha
    rc = opt_rc(a)
    kc = opt_kc(a)
    if rc <= 0 or kc <= 0 or rc == np.inf or kc == np.inf:
        raise ValueError("Invalid cutoff values computed")
    return dict(alpha=a, real_cutoff=rc, k_max=kc, error_real=real_err(rc, a), error_recip=recip_err(kc, a))
