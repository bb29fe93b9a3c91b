"""Block averaging and the GCMC energy / loading / heat-of-adsorption analysis in float64
(oracle, test infrastructure).

Restates src/kups/core/utils/block_average.py: ``compute_block_means`` (:40-84, incomplete
trailing samples dropped), ``block_average_from_blocks`` (:87-111, SEM = std(ddof=1) /
sqrt(n_blocks)) and ``block_average`` (:115-161); and ``_analyze_single_system`` of
src/kups/application/mcmc/analysis.py:82-158 (block means of U, N, U N and N N (x) N, per
block Q = (<UN> - <U><N>) cov(N)^-1 - kT, composition-weighted total) from per-step series.
"""

from __future__ import annotations

import numpy as np

from .units import BOLTZMANN_CONSTANT


def compute_block_means(data, n_blocks: int, axis: int = 0) -> np.ndarray:
    data = np.moveaxis(np.asarray(data, np.float64), axis, 0)
    size = data.shape[0] // n_blocks
    blocks = data[: size * n_blocks].reshape((n_blocks, size) + data.shape[1:]).mean(axis=1)
    return np.moveaxis(blocks, 0, axis)


def block_average_from_blocks(values, axis: int = 0):
    values = np.asarray(values, np.float64)
    n = values.shape[axis]
    with np.errstate(invalid="ignore", divide="ignore"):
        sem = np.std(values, axis=axis, ddof=1) / np.sqrt(n) if n > 1 else np.full(
            np.delete(values.shape, axis), np.nan)
    return np.mean(values, axis=axis), sem, n


def block_average(data, n_blocks: int, axis: int = 0):
    return block_average_from_blocks(compute_block_means(data, n_blocks, axis), axis)


def analyze_single_system(energy, counts, temperature: float, n_blocks: int) -> dict:
    """energy [T], counts [T, M] -> {name: (mean, sem, n_blocks)}."""
    energy = np.asarray(energy, np.float64)
    counts = np.asarray(counts, np.float64).reshape(len(energy), -1)
    u = compute_block_means(energy, n_blocks)
    n = compute_block_means(counts, n_blocks)
    un = compute_block_means(energy[:, None] * counts, n_blocks)
    nn = compute_block_means(counts[:, :, None] * counts[:, None, :], n_blocks)
    cov = nn - n[:, :, None] * n[:, None, :]
    diff = un - u[:, None] * n
    try:
        inv = np.linalg.inv(cov)
    except np.linalg.LinAlgError:  # singular count covariance: the reference's inverse gives inf / nan
        inv = np.full_like(cov, np.nan)
    hoa = np.einsum("bi,bij->bj", diff, inv) - temperature * BOLTZMANN_CONSTANT
    with np.errstate(invalid="ignore", divide="ignore"):  # a block without molecules: nan, as in the reference
        w = n / n.sum(axis=1, keepdims=True)
    return {
        "energy": block_average(energy, n_blocks),
        "loading": block_average(counts, n_blocks),
        "heat_of_adsorption": block_average_from_blocks(hoa),
        "total_heat_of_adsorption": block_average_from_blocks((hoa * w).sum(axis=1)),
    }
