"""Block averaging / GCMC analysis: the oracle against the reference's known answers
(test/core/test_block_average.py, test/application/test_mcmc_analysis.py), and the
block-sum analysis of the package against the oracle on per-step series (CPU)."""

import numpy as np
import pytest

from kups_gb300 import analysis
from oracle import analysis as oan


def test_block_average_known_answers():
    m, s, n = oan.block_average(np.arange(100.0), 10)
    assert n == 10 and m == pytest.approx(49.5)
    m, s, _ = oan.block_average(np.ones((100, 3)) * np.arange(3), 10)
    np.testing.assert_allclose(m, np.arange(3)) and np.testing.assert_allclose(s, 0, atol=1e-12)
    m, _, _ = oan.block_average(np.arange(105.0), 10)  # trailing incomplete block dropped
    assert m == pytest.approx(np.arange(100.0).mean())
    bm = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    m, s, _ = oan.block_average(np.repeat(bm, 20), 5)
    assert m == pytest.approx(3.0) and s == pytest.approx(np.std(bm, ddof=1) / np.sqrt(5))
    _, s, n = oan.block_average(np.arange(100.0), 1)
    assert n == 1 and np.isnan(s)


def test_mcmc_analysis_known_answers():
    r = oan.analyze_single_system(np.ones(200), np.tile([[2.0, 6.0], [4.0, 8.0]], (100, 1)), 300.0, 10)
    np.testing.assert_allclose(r["loading"][0], [3.0, 7.0])
    e = np.full(200, 2.0)
    c = np.tile([[3.0, 5.0]], (200, 1))
    m = oan.compute_block_means(e, 10)
    np.testing.assert_allclose(m, 2.0)
    r = oan.block_average(c, 10)
    np.testing.assert_allclose(r[0], [3.0, 5.0]) and np.testing.assert_allclose(r[1], 0, atol=1e-12)


def _series(rng, steps, n_sys):
    n = rng.poisson(6.0, (steps, n_sys)).astype(float)
    u = -0.25 * n + rng.normal(0, 0.1, (steps, n_sys))  # correlated energy and loading
    return u, n


def _sums(u, n, block):
    t, s = u.shape
    x = np.stack([u, n, u * n, n * n, u * u], -1)
    return x.reshape(t // block, block, s, 5).sum(1)


@pytest.mark.parametrize("n_blocks", [None, 8, 4])
def test_block_sum_analysis_matches_oracle_series(n_blocks):
    rng = np.random.default_rng(3)
    u, n = _series(rng, 1600, 3)
    temps = np.array([250.0, 300.0, 350.0])
    sums = _sums(u, n, 50)  # 32 device blocks of 50 steps
    res = analysis.gcmc_block_analysis(sums, 50, temps, n_blocks)
    nb = res["energy"].n_blocks
    if n_blocks is not None:
        assert nb == n_blocks
    for s in range(3):
        ref = oan.analyze_single_system(u[:, s], n[:, s], temps[s], nb)
        for key in ("energy", "loading", "heat_of_adsorption"):
            got = getattr(res[key], "mean")[s], getattr(res[key], "sem")[s]
            np.testing.assert_allclose(got[0], np.ravel(ref[key][0])[0], rtol=1e-10)
            np.testing.assert_allclose(got[1], np.ravel(ref[key][1])[0], rtol=1e-8)


def test_block_sum_analysis_rejects_uneven_merge():
    with pytest.raises(ValueError):
        analysis.gcmc_block_analysis(np.zeros((10, 2, 5)), 5, [300.0, 300.0], n_blocks=4)
