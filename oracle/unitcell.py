"""Triclinic unit-cell arithmetic in float64 (oracle, test infrastructure).

Restates src/kups/core/unitcell.py:251-380 (``TriclinicUnitCell``: ``tril`` =
[L00, L10, L11, L20, L21, L22], row convention r = f @ L), ``_wrap``
(:139-171), ``_perpendicular_lengths`` (:174-193), ``_build_lattice_vectors``
(:99-136) and src/kups/core/utils/math.py:177-239 (``triangular_3x3_matmul``,
side RIGHT => x @ L).  The products are written out term by term in a fixed
left-to-right order; the CUDA kernels use the same order so that float64
membership tests agree bit for bit.
"""

from __future__ import annotations

import numpy as np

TRIL_IDX = ((0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2))


def lattice_from_tril(tril: np.ndarray) -> np.ndarray:
    tril = np.asarray(tril, dtype=np.float64)
    L = np.zeros(tril.shape[:-1] + (3, 3))
    for k, (a, b) in enumerate(TRIL_IDX):
        L[..., a, b] = tril[..., k]
    return L


def tril_from_lattice(L: np.ndarray) -> np.ndarray:
    L = np.asarray(L, dtype=np.float64)
    return np.stack([L[..., a, b] for a, b in TRIL_IDX], axis=-1)


def lattice_from_lengths_angles(lengths, angles) -> np.ndarray:
    """src/kups/core/unitcell.py:99-136."""
    a, b, c = (float(x) for x in lengths)
    al, be, ga = (np.radians(float(x)) for x in angles)
    ca, cb, cg, sg = np.cos(al), np.cos(be), np.cos(ga), np.sin(ga)
    c2z = c * np.sqrt(1 - ca**2 - cb**2 - cg**2 + 2 * ca * cb * cg) / sg
    return np.array(
        [[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [c * cb, c * (ca - cb * cg) / sg, c2z]]
    )


def inverse_tril(tril: np.ndarray) -> np.ndarray:
    """Inverse of the lower-triangular lattice by forward substitution.

    Returns the 6 lower-triangular entries of L^-1 in ``tril`` order.
    (The reference solves L X = I with ``solve_triangular``,
    src/kups/core/utils/math.py:134-167.)
    """
    t = np.asarray(tril, dtype=np.float64)
    a, b, c, d, e, f = (t[..., k] for k in range(6))
    i00 = 1.0 / a
    i11 = 1.0 / c
    i22 = 1.0 / f
    i10 = -(b * i00) / c
    i21 = -(e * i11) / f
    i20 = -((d * i00) + (e * i10)) / f
    return np.stack([i00, i10, i11, i20, i21, i22], axis=-1)


def row_times_tril(x: np.ndarray, t: np.ndarray) -> np.ndarray:
    """x @ L for lower-triangular L given by its tril entries (broadcasting)."""
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    x0, x1, x2 = x[..., 0], x[..., 1], x[..., 2]
    y0 = (x0 * t[..., 0] + x1 * t[..., 1]) + x2 * t[..., 3]
    y1 = x1 * t[..., 2] + x2 * t[..., 4]
    y2 = x2 * t[..., 5]
    return np.stack([y0, y1, y2], axis=-1)


def to_fractional(r: np.ndarray, tril: np.ndarray) -> np.ndarray:
    return row_times_tril(r, inverse_tril(tril))


def to_cartesian(f: np.ndarray, tril: np.ndarray) -> np.ndarray:
    return row_times_tril(f, tril)


def volume(tril: np.ndarray) -> np.ndarray:
    t = np.asarray(tril, dtype=np.float64)
    return np.abs(t[..., 0] * t[..., 2] * t[..., 5])


def perpendicular_lengths(tril: np.ndarray) -> np.ndarray:
    """Face-to-face widths V/|b x c|, V/|a x c|, V/|a x b| (unitcell.py:174-193)."""
    t = np.asarray(tril, dtype=np.float64)
    L00, L10, L11, L20, L21, L22 = (t[..., k] for k in range(6))
    v = volume(t)
    bxc = np.sqrt((L11 * L22) ** 2 + (L10 * L22) ** 2 + (L10 * L21 - L11 * L20) ** 2)
    axc = np.sqrt((L00 * L22) ** 2 + (L00 * L21) ** 2)
    axb = np.abs(L00 * L11)
    return np.stack([v / bxc, v / axc, v / axb], axis=-1)


def wrap(r: np.ndarray, tril: np.ndarray) -> np.ndarray:
    """Wrap Cartesian positions into fractional [-0.5, 0.5) (unitcell.py:139-171)."""
    f = to_fractional(r, tril)
    f = np.mod(f + 0.5, 1.0) - 0.5
    return to_cartesian(f, tril)


def make_supercell(tril: np.ndarray, reps: int, positions: np.ndarray, *extra):
    """Replicate a cell ``reps`` times along each axis (unitcell.py:477-506)."""
    L = lattice_from_tril(tril)
    shifts = np.array(
        [(i, j, k) for i in range(reps) for j in range(reps) for k in range(reps)],
        dtype=np.float64,
    )
    offs = shifts @ L
    pos = (positions[None, :, :] + offs[:, None, :]).reshape(-1, 3)
    rest = [np.tile(np.asarray(e), (len(shifts),) + (1,) * (np.asarray(e).ndim - 1)) for e in extra]
    return tril_from_lattice(L * reps), pos, *rest
