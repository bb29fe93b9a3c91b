"""Local MLIAP oracle: the reference test model's energy by hand (CPU)."""

import numpy as np
import pytest

from oracle import mliap as oml


def test_two_atoms_known_answer():
    """Two atoms 2 A apart, cutoff 2.5: each gets one message 0.1 / 3 per feature, so the energy
    is 2 * 0.1 * 4 * (0.1 + 0.1 / 3)."""
    pos = np.array([[1.0, 1.0, 1.0], [3.0, 1.0, 1.0]])
    e, h, m = oml.local_mliap_energy(oml.simple_model(), pos, [0, 1], [0, 0], [[30.0, 0, 30.0, 0, 0, 30.0]], [2.5])
    np.testing.assert_allclose(m, np.full((2, 4), 0.1 / 3.0), rtol=1e-14)
    assert e[0] == pytest.approx(2 * 0.1 * 4 * (0.1 + 0.1 / 3.0), rel=1e-14)


def test_chain_of_the_reference_test():
    """Atoms on a line 3 A apart with cutoff 2.5 see no neighbour: energy = N * 0.1 * 4 * 0.1."""
    pos = np.array([[i * 3.0, 0.0, 0.0] for i in range(5)])
    e, _, m = oml.local_mliap_energy(oml.simple_model(), pos, np.zeros(5, int), np.zeros(5, int),
                                     [[30.0, 0, 30.0, 0, 0, 30.0]], [2.5])
    assert np.all(m == 0) and e[0] == pytest.approx(5 * 0.04)
