"""Energy, loading and heat of adsorption of GCMC runs from device-side block sums.

The reference logs the potential energy and particle counts of every system at every step
to HDF5 and block-averages the time series afterwards (``analyze_mcmc``,
src/kups/application/mcmc/analysis.py:82-158, with src/kups/core/utils/block_average.py).
Here ``kups_gcmc_run`` adds, after every step, U, N, U N, N^2 and U^2 of each system into a
float64 ``[S, 5]`` buffer on the device; the host reads it once per block, so no per-step
device-to-host copy is made, and the block means below equal the reference's
``compute_block_means`` of the per-step series exactly (a block here is ``block_steps``
consecutive steps; the reference's equal split of T steps into n blocks is the same thing
with ``block_steps = T // n``).

Per block b: <U>, <N>, <U N>, <N^2>; heat of adsorption (one adsorbate species)
Q_b = (<UN> - <U><N>) / (<N^2> - <N>^2) - kT; results are (mean, SEM) over blocks with
SEM = std(ddof=1) / sqrt(n_blocks) (``block_average_from_blocks``).  ``n_blocks=None``
merges adjacent device blocks by powers of two and picks the first size at which the
energy's SEM changes by less than 5 % (``optimal_block_average``'s plateau rule, on the
device blocks as the base unit).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .units import BOLTZMANN_CONSTANT

U, N, UN, NN, UU = range(5)


@dataclass
class BlockAverage:
    mean: np.ndarray
    sem: np.ndarray
    n_blocks: int


def block_average_from_blocks(values, axis: int = 0) -> BlockAverage:
    values = np.asarray(values, np.float64)
    n = values.shape[axis]
    mean = values.mean(axis=axis)
    if n < 2:
        return BlockAverage(mean, np.full(np.shape(mean), np.nan), n)
    return BlockAverage(mean, values.std(axis=axis, ddof=1) / np.sqrt(n), n)


def merge_blocks(block_sums, factor: int) -> np.ndarray:
    """Sums of `factor` adjacent blocks ([n_blocks, ...] -> [n_blocks // factor, ...]); a trailing
    incomplete group is dropped, as compute_block_means drops trailing samples."""
    b = np.asarray(block_sums, np.float64)
    m = b.shape[0] // factor
    return b[: m * factor].reshape((m, factor) + b.shape[1:]).sum(axis=1)


def _plateau_factor(block_sums, block_steps: int, min_blocks: int = 4, rtol: float = 0.05) -> int:
    n_dev = np.asarray(block_sums).shape[0]
    factors = []
    f = 1
    while n_dev // f >= min_blocks:
        factors.append(f)
        f *= 2
    if len(factors) < 2:
        return 1
    sems = []
    for f in factors:
        e = merge_blocks(np.asarray(block_sums)[..., U], f) / (block_steps * f)
        sems.append(block_average_from_blocks(e).sem)
    sems = np.asarray(sems)
    rel = np.abs(np.diff(sems, axis=0)) / (np.abs(sems[:-1]) + 1e-10)
    if rel.ndim > 1:
        rel = rel.max(axis=tuple(range(1, rel.ndim)))
    idx = np.where(rel < rtol)[0]
    return factors[idx[0] + 1] if len(idx) else factors[-1]


def gcmc_block_analysis(block_sums, block_steps: int, temperature, n_blocks: int | None = None) -> dict:
    """block_sums [n_device_blocks, S, 5] (each row the sums of `block_steps` steps) ->
    {"energy", "loading", "heat_of_adsorption", "energy_fluctuation"}: BlockAverage over
    systems (arrays of shape [S]).  With `n_blocks`, the device blocks are merged into
    `n_blocks` equal blocks (their count must divide evenly)."""
    b = np.asarray(block_sums, np.float64)
    if b.ndim != 3 or b.shape[2] != 5:
        raise ValueError("block_sums must have shape [n_blocks, S, 5]")
    if n_blocks is None:
        factor = _plateau_factor(b, block_steps)
    else:
        if n_blocks < 1 or b.shape[0] % n_blocks:
            raise ValueError(f"{b.shape[0]} device blocks cannot form {n_blocks} equal blocks")
        factor = b.shape[0] // n_blocks
    m = merge_blocks(b, factor) / (block_steps * factor)  # block means
    kt = np.asarray(temperature, np.float64) * BOLTZMANN_CONSTANT
    var_n = m[..., NN] - m[..., N] ** 2
    with np.errstate(invalid="ignore", divide="ignore"):
        q = (m[..., UN] - m[..., U] * m[..., N]) / var_n - kt
    return {
        "energy": block_average_from_blocks(m[..., U]),
        "loading": block_average_from_blocks(m[..., N]),
        "heat_of_adsorption": block_average_from_blocks(q),
        "energy_fluctuation": block_average_from_blocks(m[..., UU] - m[..., U] ** 2),
    }
