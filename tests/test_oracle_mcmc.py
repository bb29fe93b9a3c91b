"""Oracle of the Monte Carlo step (moves, muVT acceptance, step widths) and the host-side
Peng-Robinson fugacity, pinned to the reference's own known-answer tests:

* test/mcmc/test_probability.py:194-292 (exact Boltzmann ratio, temperature dependence, k_B scaling);
* test/mcmc/test_log_fugacity_ratio.py (insertion, deletion, two species with mixed changes);
* test/mcmc/test_fugacity.py (ideal limit, numpy-roots cross-check at 50 bar, binary mixtures);
* test/core/test_parameter_scheduler.py:177-360 (history, cycle, bounds, correlation);
* test/core/test_quaternion.py (identity, inverse, power, matrix, rotation of a vector);
* test/core/test_math.py:21-86 (ln(N! / M!) of the muVT ratio);
* test/core/test_position.py:77-109 (the unweighted centre the rotation move turns about);
* test/potential/test_lennard_jones.py:388-450 (global tail correction energy and pressure);
* Philox4x32-10 against the published known-answer vectors of the Random123 distribution.
"""

import math

import numpy as np
import pytest

from oracle import mcmc as om
from oracle import lennard_jones as olj
from oracle.units import BAR, BOLTZMANN_CONSTANT, PASCAL


# ----------------------------------------------------------------------------- generator
@pytest.mark.parametrize("ctr,key,expected", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_known_answers(ctr, key, expected):
    assert om.philox4x32_10(ctr, *key) == expected


def test_normals_are_standard():
    z = np.array([om.normal4(7, 3, c) for c in range(4000)]).ravel()
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1.0) < 0.03


# ----------------------------------------------------------------------------- Boltzmann ratio
T3 = np.array([300.0, 350.0, 400.0])
E3 = np.array([-100.0, -150.0, -200.0])


@pytest.mark.parametrize("delta_e", [-10.0, -5.0, 0.0, 5.0, 10.0])
def test_exact_boltzmann_ratio(delta_e):
    got = om.boltzmann_log_ratio(E3, E3 + delta_e, T3)
    np.testing.assert_allclose(got, (E3 - (E3 + delta_e)) / (T3 * BOLTZMANN_CONSTANT), rtol=1e-10)


def test_boltzmann_temperature_dependence_and_scaling():
    for t in (100.0, 1000.0):
        np.testing.assert_allclose(om.boltzmann_log_ratio(E3, E3 + 5.0, np.full(3, t)),
                                   -5.0 / (t * BOLTZMANN_CONSTANT), rtol=1e-10)
    np.testing.assert_allclose(om.boltzmann_log_ratio([0.0], [BOLTZMANN_CONSTANT], [1.0]), [-1.0], rtol=1e-15)
    np.testing.assert_allclose(om.boltzmann_log_ratio([-100.0], [-105.0], [500.0]),
                               [5.0 / (500.0 * BOLTZMANN_CONSTANT)], rtol=1e-10)


# ----------------------------------------------------------------------------- fugacity ratio
LN2 = np.log(np.array([[2.0], [2.0], [2.0]]))
VOL = np.array([1.0, 2.0, 3.0])
CNT = np.array([[0], [1], [2]])


def test_log_fugacity_ratio_insertion():
    got = om.log_fugacity_ratio(LN2, VOL, CNT, CNT + 1)
    exp = LN2[0] + np.log(VOL) + om.log_factorial_ratio(CNT[:, 0], CNT[:, 0] + 1)
    np.testing.assert_allclose(got, exp, rtol=0, atol=1e-12)
    # ln fV - ln(N + 1) written out
    np.testing.assert_allclose(got, np.log(2.0 * VOL) - np.log(CNT[:, 0] + 1.0), rtol=0, atol=1e-12)


def test_log_fugacity_ratio_deletion():
    patched = CNT - (CNT > 0)
    got = om.log_fugacity_ratio(LN2, VOL, CNT, patched)
    mask = CNT[:, 0] > 0
    exp = -(LN2[0] + np.log(VOL))[mask] + om.log_factorial_ratio(CNT[mask, 0], patched[mask, 0])
    np.testing.assert_allclose(got[mask], exp, rtol=0, atol=1e-12)
    assert got[0] == 0.0  # nothing to delete: unchanged count, zero ratio


def test_log_fugacity_ratio_two_species_mixed():
    la = np.log(np.array([[2.0, 5.0], [2.0, 5.0]]))
    vol = np.array([1.5, 0.5])
    c = np.array([[2, 3], [4, 1]])
    d = np.array([[+1, -1], [-1, +1]])
    got = om.log_fugacity_ratio(la, vol, c, c + d)
    exp = (d * (la + np.log(vol)[:, None]) + om.log_factorial_ratio(c, c + d)).sum(-1)
    np.testing.assert_allclose(got, exp, rtol=0, atol=1e-12)


def test_muvt_is_the_sum_of_both_terms():
    got = om.muvt_log_ratio(E3, E3 + 0.1, T3, LN2, VOL, CNT, CNT + 1)
    exp = om.boltzmann_log_ratio(E3, E3 + 0.1, T3) + om.log_fugacity_ratio(LN2, VOL, CNT, CNT + 1)
    np.testing.assert_allclose(got, exp, rtol=1e-15)


def test_gcmc_log_acceptance_matches_components():
    T, la, V = 298.0, -9.0, 13532.0
    for n_old, n_new, de in ((4, 5, -0.3), (4, 3, 0.2), (4, 4, 0.05), (0, 1, -0.1)):
        exp = -de / (T * BOLTZMANN_CONSTANT) + (n_new - n_old) * (la + math.log(V)) + (
            math.lgamma(n_old + 1) - math.lgamma(n_new + 1))
        assert abs(om.gcmc_log_acceptance(de, T, la, V, n_old, n_new) - exp) < 1e-12


# ----------------------------------------------------------------------------- Peng-Robinson (host code)
PC, TC, OMEGA = 7.84e6 * PASCAL, 303.75, 0.22394


def test_peng_robinson_ideal_limit():
    from kups_gb300.gcmc import peng_robinson_log_fugacity

    p = 1e-2 * BAR
    res = peng_robinson_log_fugacity(p, 300.0, [PC], [TC], [OMEGA])
    np.testing.assert_allclose(res.compressibility, [1.0], rtol=0, atol=1e-4)
    np.testing.assert_allclose(res.log_fugacity, [np.log(p)], rtol=0, atol=1e-4)


def test_peng_robinson_against_numpy_roots_at_50_bar():
    from kups_gb300.gcmc import peng_robinson_log_fugacity

    T, p = 300.0, 50.0 * BAR
    out = peng_robinson_log_fugacity(p, T, [PC], [TC], [OMEGA])
    pr, tr = p / PC, T / TC
    m = 0.37464 + 1.54226 * OMEGA - 0.26992 * OMEGA**2
    A = 0.45724 * pr / tr**2 * (1 + m * (1 - np.sqrt(tr))) ** 2
    B = 0.0778 * pr / tr
    roots = np.roots([1.0, -(1.0 - B), A - 3.0 * B**2 - 2.0 * B, -(A * B - B**2 - B**3)])
    Z = roots[np.isclose(roots.imag, 0.0, atol=1e-12)].real.max()
    sq2 = np.sqrt(2.0)
    ln_phi = Z - 1.0 - np.log(Z - B) - A / (2.0 * sq2 * B) * np.log((Z + (1 + sq2) * B) / (Z + (1 - sq2) * B))
    np.testing.assert_allclose(out.compressibility, [Z], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(out.log_fugacity, [ln_phi + np.log(p)], rtol=1e-10, atol=1e-10)


def test_peng_robinson_binary_mixtures():
    from kups_gb300.gcmc import peng_robinson_log_fugacity

    two = lambda v: [v, v]
    y = np.array([0.25, 0.75])
    low = peng_robinson_log_fugacity(1e-2 * BAR, 300.0, two(PC), two(TC), two(OMEGA), y, np.zeros((2, 2)))
    np.testing.assert_allclose(low.compressibility, np.ones(2), rtol=0, atol=1e-4)
    np.testing.assert_allclose(low.log_fugacity, np.log(y * 1e-2 * BAR), rtol=0, atol=2e-4)
    p = 50.0 * BAR
    mix = peng_robinson_log_fugacity(p, 300.0, two(PC), two(TC), two(OMEGA), [1.0, 0.0], np.zeros((2, 2)))
    pure = peng_robinson_log_fugacity(p, 300.0, [PC], [TC], [OMEGA])
    np.testing.assert_allclose(mix.log_fugacity[0], pure.log_fugacity[0], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(mix.compressibility[0], pure.compressibility[0], rtol=1e-10, atol=1e-10)


# ----------------------------------------------------------------------------- step-width scheduler
def _run(sched, values):
    for v in values:
        sched(v)
    return sched.value


def test_scheduler_history_and_cycle():
    a = om.AcceptanceScheduler(1.0, 2.0, 0.5, 0.1, lower=None, history_length=5)
    b = om.AcceptanceScheduler(2.0, 2.0, 0.5, 0.1, lower=None, history_length=5)
    a(0.3), b(0.7)
    assert (a.value, b.value, a.index, b.index) == (1.0, 2.0, 1, 1)
    np.testing.assert_allclose(_run(a, [0.3] * 4), 0.5)
    np.testing.assert_allclose(_run(b, [0.7] * 4), 4.0)
    assert a.index == 0 and b.index == 0
    c = om.AcceptanceScheduler(1.0, 2.0, 0.5, 0.1, lower=None, history_length=5)
    for v in (0.1, 0.3, 0.5, 0.7, 0.9):
        c(v)
    np.testing.assert_array_equal(c.history, [0.1, 0.3, 0.5, 0.7, 0.9])


def test_scheduler_edge_cases_and_bounds():
    mk = lambda v, m, t, tol, lo=None, up=None, n=5: om.AcceptanceScheduler(v, m, t, tol, lo, up, n)
    for v in (1.0, 2.0):
        np.testing.assert_allclose(_run(mk(v, 2.0, 0.5, 0.1), [0.5] * 5), v)
        np.testing.assert_allclose(_run(mk(v, 2.0, 0.5, 0.1), [0.0] * 5), v * 0.5)
        np.testing.assert_allclose(_run(mk(v, 2.0, 0.5, 0.1), [1.0] * 5), v * 2.0)
    np.testing.assert_allclose(_run(mk(1.5, 1.5, 0.6, 0.1, n=3), [0.4] * 3), 1.0)
    np.testing.assert_allclose([_run(mk(v, 3.0, 0.5, 0.05, up=2.5, n=4), [0.9] * 4) for v in (1.0, 2.0)],
                               [2.5, 2.5])
    np.testing.assert_allclose([_run(mk(v, 4.0, 0.6, 0.05, lo=lo), [0.0] * 5) for v, lo in ((1.0, 0.8), (2.0, 1.5))],
                               [0.8, 1.5])
    np.testing.assert_allclose([_run(mk(1.0, 2.0, 0.5, 0.05, 0.9, 1.5, 3), [0.9] * 3),
                                _run(mk(5.0, 2.0, 0.5, 0.05, 4.0, 6.0, 3), [0.1] * 3)], [1.5, 4.0])


def test_scheduler_correlation():
    neg = [om.AcceptanceScheduler(v, 3.0, 0.5, 0.1, None, None, 5) for v in (1.0, 2.0)]
    pos = [om.AcceptanceScheduler(v, 3.0, 0.5, 0.1, None, None, 5, positive=True) for v in (1.0, 2.0)]
    np.testing.assert_allclose([_run(s, [0.3] * 5) for s in neg], [1.0 / 3.0, 2.0 / 3.0])
    np.testing.assert_allclose([_run(s, [0.3] * 5) for s in pos], [3.0, 6.0])


# ----------------------------------------------------------------------------- quaternions
def test_quaternion_identity_inverse_and_product():
    q = np.array([0.5, 0.5, 0.5, 0.5])
    inv = q * np.array([1, -1, -1, -1])
    np.testing.assert_array_equal(inv, [0.5, -0.5, -0.5, -0.5])
    np.testing.assert_allclose(om.qmul(q, inv), [1, 0, 0, 0], atol=1e-12)
    np.testing.assert_allclose(om.qmul([1.0, 0, 0, 0], q), q)
    q2 = np.array([0.6, 0.8, 0.0, 0.0])
    np.testing.assert_allclose(om.qmul(q2, q2 * np.array([1, -1, -1, -1])), [1, 0, 0, 0], atol=1e-12)


def test_quaternion_power():
    q = np.array([0.6, 0.8, 0.0, 0.0])
    np.testing.assert_allclose(om.qpow(q, 1.0), q, atol=1e-6)
    np.testing.assert_allclose(om.qpow(q, 0.0), [1, 0, 0, 0], atol=1e-6)
    sq = om.qpow(q, 2.0)
    np.testing.assert_allclose(sq, om.qmul(q, q), atol=1e-12)
    small = np.array([math.cos(5e-11), math.sin(5e-11), 0.0, 0.0])
    for p in (0.0, 0.5, 1.0, 2.0):
        r = om.qpow(small, p)
        assert np.all(np.isfinite(r)) and abs(np.linalg.norm(r) - 1.0) < 1e-12
    np.testing.assert_allclose(om.qpow([1.0, 0, 0, 0], 0.7), [1, 0, 0, 0], atol=1e-12)


def test_quaternion_matrix_and_rotation():
    for seed in range(5):
        rng = np.random.default_rng(seed)
        R = om.quat_matrix(om.shoemake(*rng.uniform(0, 1, 3)))
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
        np.testing.assert_allclose(np.linalg.det(R), 1.0, atol=1e-12)
    half = math.pi / 4  # 90 degrees about z
    q = np.array([math.cos(half), 0.0, 0.0, math.sin(half)])
    np.testing.assert_allclose(om.rotate([1.0, 0.0, 0.0], q), [0.0, 1.0, 0.0], atol=1e-12)
    np.testing.assert_array_equal(om.rotate([1.0, 2.0, 3.0], [1.0, 0, 0, 0]), [1.0, 2.0, 3.0])


def test_shoemake_is_uniform_on_rotations():
    # the rotated x axis of a uniform rotation is uniform on the sphere: E[x] = 0, E[x x^T] = I / 3
    v = np.array([om.rotate([1.0, 0, 0], om.shoemake(*np.random.default_rng(i).uniform(0, 1, 3)))
                  for i in range(3000)])
    assert np.abs(v.mean(0)).max() < 0.05
    np.testing.assert_allclose(v.T @ v / len(v), np.eye(3) / 3, atol=0.03)


# ----------------------------------------------------------------------------- LJ global tail correction
def test_global_tail_correction_known_answer():
    sigma = np.array([[1.0, 1.2], [1.2, 1.0]])
    epsilon = np.array([[1.0, 0.8], [0.8, 1.0]])
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0]])
    counts = np.array([[1.0, 1.0]])
    got = olj.tail_correction_energy(counts, tril, sigma, epsilon, [12.0], np.ones((2, 2), bool))
    t1 = (sigma / 12.0) ** 3
    target = (8 / 3 * np.pi * (np.outer([1, 1], [1, 1]) / 1000.0) * epsilon * sigma**3 * (t1**3 / 3 - t1)).sum()
    assert got.shape == (1,)
    np.testing.assert_allclose(got, [target], rtol=1e-6)
    for mask in (np.ones((2, 2), bool), np.eye(2, dtype=bool)):
        p = olj.tail_correction_pressure(counts, tril, sigma, epsilon, [12.0], mask)
        assert p.shape == (1,) and np.isfinite(p[0])


# ----------------------------------------------------------------------------- the replayed moves
def test_proposals_keep_molecule_geometry():
    from oracle.unitcell import lattice_from_lengths_angles, tril_from_lattice

    L = lattice_from_lengths_angles([12.0, 12.0, 13.0], [90, 90, 120])
    tril = tril_from_lattice(L)
    motif = np.array([[0.0, 0, 0], [1.16, 0, 0], [-1.16, 0, 0]])
    mols = np.stack([motif + np.array([1.0, 2.0, 3.0]), motif + np.array([5.5, 5.9, 6.4])])
    d0 = np.linalg.norm(motif[1] - motif[2])
    for kind in range(5):
        for c in range(20):
            mol, new, has_old = om.propose(3, c, 1, kind, 2, mols, motif, 0.4, tril)
            if kind == 4:
                assert has_old and new is None and 0 <= mol < 2
                continue
            f = new @ np.linalg.inv(L)
            assert np.all(f >= -0.5 - 1e-12) and np.all(f < 0.5 + 1e-12)
            d = new[1] - new[2]
            fd = d @ np.linalg.inv(L)
            d = (fd - np.round(fd)) @ L
            np.testing.assert_allclose(np.linalg.norm(d), d0, atol=1e-9)


def test_log_factorial_ratio_known_answers():
    """test/core/test_math.py:21-86: ln(N! / M!) of scalars, equal and swapped arguments, zeros,
    large counts, vectors and broadcasting."""
    lfr = om.log_factorial_ratio
    np.testing.assert_allclose(lfr(np.array([5]), np.array([3])), np.log(5 * 4), rtol=1e-10)
    np.testing.assert_allclose(lfr(np.array([4]), np.array([4])), [0.0], atol=1e-15)
    np.testing.assert_allclose(lfr(np.array([3]), np.array([5])), -np.log(5 * 4), rtol=1e-10)
    np.testing.assert_allclose(lfr(np.array([0]), np.array([0])), [0.0], atol=1e-15)
    np.testing.assert_allclose(lfr(np.array([3]), np.array([0])), np.log(6), rtol=1e-10)
    np.testing.assert_allclose(lfr(np.array([100]), np.array([95])), np.sum(np.log(np.arange(96, 101))), rtol=1e-10)
    np.testing.assert_allclose(lfr(np.array([5, 4, 10]), np.array([3, 4, 7])),
                               [np.log(5 * 4), 0.0, np.log(10 * 9 * 8)], rtol=1e-10, atol=1e-15)
    np.testing.assert_allclose(lfr(np.array([[5, 6], [7, 8]]), np.array([3, 4])),
                               [[np.log(5 * 4), np.log(6 * 5)], [np.log(7 * 6 * 5 * 4), np.log(8 * 7 * 6 * 5)]],
                               rtol=1e-10)
    np.testing.assert_allclose(lfr(np.array([7]), np.array([4])), -lfr(np.array([4]), np.array([7])), rtol=1e-10)


def test_atom_mean_known_answers():
    """The rotation centre: ``center_of_mass`` with equal weights (test/core/test_position.py:77-109):
    plain means, a pair across the cell boundary, and a single atom (its wrapped position)."""
    def mean(pos, side):
        L = np.eye(3) * side
        return om.atom_mean(np.asarray(pos, np.float64), L, np.linalg.inv(L))

    np.testing.assert_allclose(mean([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], 4.0), [0.5, 0.0, 0.0], atol=1e-10)
    np.testing.assert_allclose(mean([[0.0, 1.0, 0.0], [1.0, 1.0, 0.0]], 6.0), [0.5, 1.0, 0.0], atol=1e-10)
    np.testing.assert_allclose(mean([[0.1, 0.0, 0.0], [1.9, 0.0, 0.0]], 2.0), [0.0, 0.0, 0.0], atol=1e-10)
    np.testing.assert_allclose(mean([[1.0, 2.0, 3.0]], 4.0), [1.0, -2.0, -1.0], atol=1e-10)
    np.testing.assert_allclose(mean([[4.0, 5.0, 6.0]], 6.0), [-2.0, -1.0, 0.0], atol=1e-10)


def test_tail_change_as_a_quadratic_in_the_molecule_count():
    """The GCMC kernel adds the tail correction's change of an exchange as b dN + c d(N^2), with
    b = sum_ab coef_ab (f_a m_b + m_a f_b) and c = sum_ab coef_ab m_a m_b (f: host species
    counts, m: one molecule's); this equals the oracle's tail energy before and after."""
    from kups_gb300.gcmc import tail_coefficients
    from oracle import lennard_jones as olj
    from oracle import unitcell as ouc

    rng = np.random.default_rng(0)
    T = 6
    sig_i, eps_i = rng.uniform(2.5, 3.5, T), rng.uniform(0.0, 0.01, T)
    eps_i[2] = 0.0  # a species without dispersion (masked)
    sigma = 0.5 * (sig_i[:, None] + sig_i[None, :])
    epsilon = np.sqrt(eps_i[:, None] * eps_i[None, :])
    tril = ouc.tril_from_lattice(ouc.lattice_from_lengths_angles([25.0, 25.0, 25.0], [90, 90, 120]))
    vol = float(ouc.volume(tril))
    rc = 12.0
    coef = tail_coefficients(sigma, epsilon, rc, vol)
    f = np.array([500.0, 700.0, 300.0, 500.0, 0.0, 0.0])
    m = np.array([0.0, 0.0, 0.0, 0.0, 1.0, 2.0])
    b = float(np.sum(coef * (f[:, None] * m[None, :] + m[:, None] * f[None, :])))
    c = float(np.sum(coef * (m[:, None] * m[None, :])))
    for n_old, n_new in ((0, 1), (7, 8), (8, 7), (120, 121)):
        e = [olj.tail_correction_energy((f + n * m)[None], tril[None], sigma, epsilon, np.array([rc]))[0]
             for n in (n_old, n_new)]
        quad = b * (n_new - n_old) + c * (n_new * n_new - n_old * n_old)
        np.testing.assert_allclose(quad, e[1] - e[0], rtol=1e-9, atol=1e-12)
