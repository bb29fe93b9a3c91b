"""Oracle of the CSVR thermostat, the virial stress / instantaneous pressure and the
stochastic cell-rescaling barostat (CPU), pinned to the reference's known answers in
test/md/test_integrators.py."""

import numpy as np

from oracle import md as omd


def test_instantaneous_pressure_known_stress():
    """test_integrators.py:700-705: K = 10, sigma = 5 I, V = 125 -> 2K / 3V + 15 / 3."""
    p = omd.instantaneous_pressure([10.0], np.eye(3)[None] * 5.0, [[5.0, 0, 5.0, 0, 0, 5.0]])
    np.testing.assert_allclose(p, [20.0 / 375.0 + 5.0], rtol=1e-12)


def test_virial_stress_convention_harmonic():
    """test_integrators.py:708-745: forces -k r in a 5 A box, no cell gradient;
    P = 2K / 3V + Tr(sum_i r_i (x) F_i) / 3V."""
    pos = np.array([[1.0, 0.5, -0.3], [-0.5, 1.2, 0.1], [0.3, -0.7, 0.8], [-0.2, 0.4, -0.6], [0.6, -0.1, 0.2]])
    frc = -pos
    mom = np.full_like(pos, 0.5)
    tril = np.array([[5.0, 0, 5.0, 0, 0, 5.0]])
    stress = omd.virial_stress(pos, -frc, np.zeros(5, int), tril, np.zeros((1, 6)))
    ke = 0.5 * np.sum(mom**2)
    expected = 2 * ke / (3 * 125.0) + np.trace(pos.T @ frc) / (3 * 125.0)
    np.testing.assert_allclose(omd.instantaneous_pressure([ke], stress, tril), [expected], rtol=1e-12)


def test_csvr_limits():
    """tau -> infinity leaves momenta unchanged; kT = 0 scales them by sqrt(exp(-dt / tau));
    E[alpha^2] = c1 + (1 - c1) K_target / K (the mean of R1^2 + R2 is N_dof)."""
    rng = np.random.default_rng(0)
    n = 7
    mom = rng.normal(size=(n, 3))
    masses = rng.uniform(1, 3, n)
    sysi = np.zeros(n, int)
    out = omd.csvr_scale(mom, masses, sysi, 1, [0.1], [300.0], [np.inf], [0.7], [5.0])
    np.testing.assert_array_equal(out, mom)
    out = omd.csvr_scale(mom, masses, sysi, 1, [0.1], [0.0], [0.5], [0.7], [5.0])
    np.testing.assert_allclose(out, mom * np.sqrt(np.exp(-0.2)), rtol=1e-14)
    dof = 3 * n - 3
    k0 = omd.kinetic_energy(mom, masses, sysi, 1)[0]
    r1 = rng.normal(size=20000)
    r2 = rng.chisquare(dof - 1, size=20000)
    k1 = [omd.kinetic_energy(omd.csvr_scale(mom, masses, sysi, 1, [0.1], [300.0], [0.5], [a], [b]), masses, sysi,
                             1)[0] for a, b in zip(r1[:2000], r2[:2000])]
    c1 = np.exp(-0.2)
    kt = dof * 300.0 * omd.BOLTZMANN_CONSTANT / 2
    assert abs(np.mean(k1) - (c1 * k0 + (1 - c1) * kt)) < 4 * np.std(k1) / np.sqrt(len(k1))


def test_cell_rescale_factor_deterministic_and_clipped():
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0], [10.0, 0, 10.0, 0, 0, 10.0]])
    mu = omd.cell_rescale_factor(np.array([2e-3, 1e3]), tril, [1.0, 1.0], [0.0, 0.0], [1e-3, 0.0], [10.0, 1.0],
                                 [5.0, 5.0], [0.9, 0.9], [0.3, 0.3])
    np.testing.assert_allclose(mu[0], np.exp(1.0 / 10.0 * 5.0 * 1e-3 / 3.0), rtol=1e-14)
    assert mu[1] == 1.0 / 0.9


def test_kinetic_energy_known_answers():
    """test_integrators.py:678-686: KE = p^2 / 2m per particle, summed per system here."""
    ke = omd.kinetic_energy(np.array([[1.0, 0.0, 0.0], [3.0, 4.0, 0.0]]), np.array([1.0, 2.0]),
                            np.array([0, 1]), 2)
    np.testing.assert_allclose(ke, [0.5, 6.25], rtol=1e-15)
