"""Oracle unit-cell arithmetic (row a1) against the reference's known answers
(test/core/test_unitcell.py: wrap :60-123, volume / inverse :23-58 and :157-173, perpendicular
lengths :175-223) and against numpy's general 3 x 3 algebra on random triclinic cells."""

import numpy as np

from oracle import unitcell as ouc


def _tril(vecs):
    return ouc.tril_from_lattice(np.asarray(vecs, np.float64))


def test_wrap_known_answers():
    # single point, unit cube (:63-65)
    np.testing.assert_allclose(ouc.wrap(np.array([1.5, -0.7, 2.3]), _tril(np.eye(3))), [-0.5, 0.3, 0.3],
                               atol=1e-10)
    # several points, cube of side 2 (:68-71)
    r = np.array([[3.0, 1.0, -1.0], [-1.0, 4.0, 0.5], [0.0, 0.0, 0.0]])
    expected = np.array([[-1.0, -1.0, -1.0], [-1.0, 0.0, 0.5], [0.0, 0.0, 0.0]])
    np.testing.assert_allclose(ouc.wrap(r, _tril(2.0 * np.eye(3))), expected, atol=1e-10)
    # the half-open interval: +0.5 and -0.5 both land on -0.5 (:74-91)
    r = np.array([[0.5, 0.0, 0.0], [-0.5, 0.0, 0.0], [0.0, 0.5, 0.0], [0.0, -0.5, 0.0]])
    expected = np.array([[-0.5, 0.0, 0.0], [-0.5, 0.0, 0.0], [0.0, -0.5, 0.0], [0.0, -0.5, 0.0]])
    np.testing.assert_allclose(ouc.wrap(r, _tril(np.eye(3))), expected, atol=1e-10)


def test_wrap_across_coordinate_spaces():
    t = _tril(2.0 * np.eye(3))
    # real -> fractional (:97-104)
    f = ouc.to_fractional(ouc.wrap(np.array([1.0, 3.0, -1.0]), t), t)
    np.testing.assert_allclose(f, [-0.5, -0.5, -0.5], atol=1e-10)
    # fractional -> real (:106-113)
    f = np.mod(np.array([1.2, -0.8, 0.3]) + 0.5, 1.0) - 0.5
    np.testing.assert_allclose(ouc.to_cartesian(f, t), [0.4, 0.4, 0.6], atol=1e-6)
    # fractional -> fractional, unit cube (:116-123)
    np.testing.assert_allclose(np.mod(np.array([1.7, -1.3, 0.8]) + 0.5, 1.0) - 0.5, [-0.3, -0.3, -0.2], atol=1e-6)


def test_volume_and_inverse_known_answers():
    # identity, orthorhombic and sheared lower-triangular lattices (:23-51, :157-173)
    for vecs, vol in ((np.eye(3), 1.0), (np.diag([2.0, 3.0, 4.0]), 24.0),
                      ([[1.0, 0.0, 0.0], [0.5, 1.0, 0.0], [0.0, 0.5, 1.0]], 1.0),
                      (np.diag([1.0, 2.0, 3.0]), 6.0)):
        t = _tril(vecs)
        np.testing.assert_allclose(ouc.volume(t), vol, rtol=1e-10)
        inv = ouc.lattice_from_tril(ouc.inverse_tril(t))
        np.testing.assert_allclose(inv, np.linalg.inv(np.asarray(vecs, np.float64)), atol=1e-12)
    np.testing.assert_allclose(ouc.lattice_from_tril(ouc.inverse_tril(_tril(np.diag([2.0, 3.0, 4.0])))),
                               np.diag([0.5, 1.0 / 3.0, 0.25]), rtol=1e-12)


def test_perpendicular_lengths_known_answers():
    np.testing.assert_allclose(ouc.perpendicular_lengths(_tril(5.0 * np.eye(3))), [5.0, 5.0, 5.0], rtol=1e-10)
    np.testing.assert_allclose(ouc.perpendicular_lengths(_tril(np.diag([2.0, 3.0, 4.0]))), [2.0, 3.0, 4.0],
                               rtol=1e-10)
    vecs = np.array([[1.0, 0.0, 0.0], [0.5, 1.0, 0.0], [0.0, 0.0, 1.0]])  # (:189-201)
    a, b, c = vecs
    v = abs(np.linalg.det(vecs))
    expected = [v / np.linalg.norm(np.cross(b, c)), v / np.linalg.norm(np.cross(a, c)),
                v / np.linalg.norm(np.cross(a, b))]
    np.testing.assert_allclose(ouc.perpendicular_lengths(_tril(vecs)), expected, rtol=1e-10)
    assert np.all(ouc.perpendicular_lengths(_tril([[1.0, 0, 0], [0.5, 1.0, 0], [0.2, 0.3, 1.0]])) > 0)
    batched = ouc.perpendicular_lengths(np.stack([_tril(np.diag([2.0, 3.0, 4.0])), _tril(5.0 * np.eye(3))]))
    assert batched.shape == (2, 3)
    np.testing.assert_allclose(batched, [[2.0, 3.0, 4.0], [5.0, 5.0, 5.0]], rtol=1e-10)


def test_random_triclinic_cells_against_general_algebra():
    rng = np.random.default_rng(0)
    for _ in range(50):
        lengths = rng.uniform(5.0, 30.0, 3)
        angles = rng.uniform(60.0, 120.0, 3)
        L = ouc.lattice_from_lengths_angles(lengths, angles)
        if not np.all(np.isfinite(L)):
            continue
        t = ouc.tril_from_lattice(L)
        np.testing.assert_allclose(ouc.volume(t), abs(np.linalg.det(L)), rtol=1e-12)
        np.testing.assert_allclose(ouc.lattice_from_tril(ouc.inverse_tril(t)), np.linalg.inv(L), rtol=1e-10,
                                   atol=1e-14)
        a, b, c = L
        v = abs(np.linalg.det(L))
        np.testing.assert_allclose(ouc.perpendicular_lengths(t),
                                   [v / np.linalg.norm(np.cross(b, c)), v / np.linalg.norm(np.cross(a, c)),
                                    v / np.linalg.norm(np.cross(a, b))], rtol=1e-12)
        r = rng.normal(0.0, 40.0, (20, 3))
        w = ouc.wrap(r, t)
        f = w @ np.linalg.inv(L)
        assert np.all(f >= -0.5 - 1e-12) and np.all(f < 0.5 + 1e-12)
        np.testing.assert_allclose(((r - w) @ np.linalg.inv(L)), np.round((r - w) @ np.linalg.inv(L)), atol=1e-9)
