"""The observables oracle against the reference's known answers
(test/observables/test_stress.py:72-190) and the molecular stress's own properties."""

import numpy as np
import pytest

from oracle import observables as ob
from oracle.unitcell import lattice_from_tril, wrap

CUBE = lambda b: np.array([[b, 0.0, b, 0.0, 0.0, b]])


@pytest.mark.parametrize("G,box,expected", [
    (np.zeros(6), 1.0, np.zeros((3, 3))),
    (np.array([2.0, 0, 2.0, 0, 0, 2.0]), 3.0, -2.0 * np.eye(3) / 27.0),
    (np.array([1.0, 3.0, 4.0, 0, 0, 5.0]), 2.0, -np.array([[1.0, 0, 0], [3.0, 4.0, 0], [0, 0, 5.0]]) / 8.0),
])
def test_lattice_stress_known_answers(G, box, expected):
    np.testing.assert_allclose(ob.lattice_stress(CUBE(box), G[None])[0], expected, rtol=1e-12, atol=1e-15)


def test_virial_stress_known_answers():
    # gradients = positions, cube of side 2: -(r0 r0^T + r1 r1^T) / 8
    r = np.array([[1.0, 0, 0], [0, 1.0, 0]])
    got = ob.virial_stress(r, r, np.zeros(2, int), CUBE(2.0), np.zeros((1, 6)))[0]
    np.testing.assert_allclose(got, -(np.outer(r[0], r[0]) + np.outer(r[1], r[1])) / 8.0, rtol=1e-12)
    # single particle at the origin: zero
    assert not ob.virial_stress(np.zeros((1, 3)), np.zeros((1, 3)), [0], CUBE(1.0), np.zeros((1, 6))).any()
    r = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]])
    got = ob.virial_stress(r, r, np.zeros(2, int), CUBE(1.0), np.zeros((1, 6)))[0]
    np.testing.assert_allclose(got, -(np.outer(r[0], r[0]) + np.outer(r[1], r[1])), rtol=1e-12)
    # lattice-gradient term: h = 2I, dU/dh = 3I: -6I / 8
    got = ob.virial_stress(np.zeros((1, 3)), np.zeros((1, 3)), [0], CUBE(2.0), np.array([[3.0, 0, 3.0, 0, 0, 3.0]]))
    np.testing.assert_allclose(got[0], -np.eye(3) * 6.0 / 8.0, rtol=1e-12)


def test_virial_stress_orientation_follows_the_reference_broadcast():
    """stress.py:77 sums position_gradients[:, None] * positions[..., None]: [a, b] = r_a g_b."""
    rng = np.random.default_rng(0)
    r, g = rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    expected = -(g[:, None] * r[..., None]).sum(0) / 8.0
    np.testing.assert_allclose(ob.virial_stress(r, g, np.zeros(5, int), CUBE(2.0), np.zeros((1, 6)))[0], expected,
                               rtol=1e-12)


def test_symmetric_positions_give_symmetric_stress():
    r = np.array([[0.25, 0.25, 0.25], [-0.25, -0.25, -0.25]])
    s = ob.virial_stress(r, r, np.zeros(2, int), CUBE(2.0), np.zeros((1, 6)))[0]
    np.testing.assert_allclose(s, s.T, atol=1e-15)
    np.testing.assert_allclose(ob.lattice_stress(CUBE(2.0), np.zeros((1, 6))), 0.0)


def _molecules(rng, tril, n_mol, size=3, spread=0.8):
    """Rigid-looking molecules around random centres, atoms wrapped one by one (so that
    molecules straddle the cell faces)."""
    L = lattice_from_tril(tril)
    centres = rng.uniform(-0.5, 0.5, (n_mol, 3)) @ L
    pos = (centres[:, None, :] + rng.normal(scale=spread, size=(n_mol, size, 3))).reshape(-1, 3)
    return wrap(pos, tril[None]), np.repeat(np.arange(n_mol), size)


def test_single_atom_groups_give_the_symmetrised_atomic_stress():
    rng = np.random.default_rng(1)
    tril = np.array([[9.0, 1.0, 8.0, -0.5, 0.7, 10.0]])
    pos = wrap(rng.uniform(-5, 5, (20, 3)), tril)
    g = rng.normal(size=(20, 3))
    dt = rng.normal(size=(1, 6))
    atomic = ob.virial_stress(pos, g, np.zeros(20, int), tril, dt)[0]
    mol = ob.molecular_virial_stress(pos, g, np.zeros(20, int), np.arange(20), 20, tril, dt)[0]
    L, G = lattice_from_tril(tril[0]), lattice_from_tril(dt[0])
    V = abs(np.linalg.det(L))
    A = -atomic * V - L.T @ G  # sum r (x) g
    np.testing.assert_allclose(mol, (-0.5 * (A + A.T) - L.T @ G) / V, rtol=1e-10, atol=1e-12)


def test_whole_molecules_use_their_mean_position():
    """Molecules whose atoms and mean lie well inside the cell: w_i is the plain mean."""
    rng = np.random.default_rng(2)
    tril = np.array([[12.0, 0.5, 11.0, -1.0, 0.3, 13.0]])
    L = lattice_from_tril(tril[0])
    centres = rng.uniform(-0.3, 0.3, (10, 3)) @ L
    pos = (centres[:, None, :] + rng.normal(scale=0.3, size=(10, 3, 3))).reshape(-1, 3)
    grp = np.repeat(np.arange(10), 3)
    g = rng.normal(size=pos.shape)
    dt = rng.normal(size=(1, 6))
    mean = pos.reshape(10, 3, 3).mean(1)
    A = np.einsum("ma,mb->ab", mean, g.reshape(10, 3, 3).sum(1))
    G = lattice_from_tril(dt[0])
    expected = (-0.5 * (A + A.T) - L.T @ G) / abs(np.linalg.det(L))
    got = ob.molecular_virial_stress(pos, g, np.zeros(30, int), grp, 10, tril, dt)[0]
    np.testing.assert_allclose(got, expected, rtol=1e-10, atol=1e-13)


def test_molecular_stress_does_not_depend_on_the_anchor_atom():
    """Molecules straddling the cell faces; reversing the atoms of every molecule changes
    the anchor (first atom) and nothing else."""
    rng = np.random.default_rng(3)
    tril = np.array([[12.0, 0.5, 11.0, -1.0, 0.3, 13.0]])
    pos, grp = _molecules(rng, tril[0], 12)
    g = rng.normal(size=pos.shape)
    dt = rng.normal(size=(1, 6))
    base = ob.molecular_virial_stress(pos, g, np.zeros(len(pos), int), grp, 12, tril, dt)
    order = np.arange(len(pos)).reshape(12, 3)[:, ::-1].reshape(-1)
    again = ob.molecular_virial_stress(pos[order], g[order], np.zeros(len(pos), int), grp[order], 12, tril, dt)
    np.testing.assert_allclose(again, base, rtol=1e-10, atol=1e-13)


def test_pressure_helpers():
    tril = CUBE(2.0)
    s = np.diag([3.0, 6.0, 9.0])[None]
    np.testing.assert_allclose(ob.pressure_from_stress(s), [6.0])
    np.testing.assert_allclose(ob.instantaneous_pressure([12.0], s, tril), [2 * 12.0 / 24.0 + 6.0])
    np.testing.assert_allclose(ob.ideal_gas_pressure([10], [300.0], tril), [10 * ob.BOLTZMANN_CONSTANT * 300.0 / 8.0])
