"""Bonded-term oracle against the reference's known answers
(test/potential/test_harmonic.py, test/potential/classical/test_{morse,cosine_angle,
dihedral,inversion}.py) and its gradients against total-energy finite differences (CPU)."""

import math

import numpy as np
import pytest

from oracle import bonded as ob

BOX = np.array([[20.0, 0, 20.0, 0, 0, 20.0]])


def energy(kind, pos, row, order):
    T = 1
    table = np.asarray(row, np.float64).reshape((T,) * order + (-1,)).reshape(1, -1)
    e, _, _ = ob.bonded(kind, pos, np.zeros(len(pos), int), np.zeros(len(pos), int), BOX, table, T,
                        np.arange(order)[None], np.zeros((1, order - 1, 3)))
    return e[0]


def dihedral_positions(phi):
    """i, j, k fixed; l rotated about the j-k axis by phi - pi from its trans position."""
    i, j, k = np.zeros(3), np.array([1.0, 0, 0]), np.array([1.5, 1.0, 0])
    axis = (k - j) / np.linalg.norm(k - j)
    t = np.array([2.5, 1.0, 0]) - k
    a = phi - np.pi
    rot = t * np.cos(a) + np.cross(axis, t) * np.sin(a) + axis * axis.dot(t) * (1 - np.cos(a))
    return np.stack([i, j, k, k + rot])


def test_dihedral_known_answers():
    assert energy("dihedral", dihedral_positions(np.pi), [2.0, 3.0, np.pi], 4) == pytest.approx(0.0, abs=1e-10)
    assert energy("dihedral", dihedral_positions(0.0), [2.0, 3.0, np.pi], 4) == pytest.approx(2.0, abs=1e-10)
    assert energy("dihedral", dihedral_positions(np.pi / 2), [2.0, 3.0, np.pi], 4) == pytest.approx(1.0, abs=1e-10)
    for phi0_deg, n in [(180, 3), (180, 2), (0, 6), (60, 3)]:
        phi0 = math.radians(phi0_deg)
        assert energy("dihedral", dihedral_positions(phi0), [2.0, n, phi0], 4) == pytest.approx(0.0, abs=1e-10)


def test_cosine_angle_known_answers():
    for deg, exp in ((90, (0.25, 0.0, 0.25)), (120, (0.5, 2 / 3, 1 / 3))):
        np.testing.assert_allclose(ob.cosine_coefficients(math.radians(deg)), exp, atol=1e-12)
    for deg in (90, 120, 180):
        t = math.radians(deg)
        pos = np.array([[0, 0, 0], [1.0, 0, 0], [math.cos(t), math.sin(t), 0]])
        assert energy("cosine_angle", pos, [t, 3.0, math.radians(5)], 3) == pytest.approx(0.0, abs=1e-10)


def inversion_positions(h):
    return np.array([[0.0, 0.0, h], [1.0, 0.0, 0.0], [-0.5, 0.866025, 0.0], [-0.5, -0.866025, 0.0]])


def inversion_omega(h):
    rji, rjk, rjl = np.array([1.0, 0, -h]), np.array([-0.5, 0.866025, -h]), np.array([-0.5, -0.866025, -h])
    n = np.cross(rjk, rjl)
    return np.arcsin(np.clip(rji.dot(n / np.linalg.norm(n)) / np.linalg.norm(rji), -1, 1))


def test_inversion_known_answers():
    assert energy("inversion", inversion_positions(0.0), [0.0, 10.0], 4) == pytest.approx(0.0, abs=1e-10)
    assert energy("inversion", inversion_positions(0.2), [0.0, 10.0], 4) == pytest.approx(
        10.0 * (1 - math.cos(inversion_omega(0.2))), rel=1e-7)
    w0 = math.radians(30.0)
    assert energy("inversion", inversion_positions(0.0), [w0, 22.0], 4) == pytest.approx(22.0, rel=1e-9)
    c2 = 1 / (4 * math.sin(w0) ** 2)
    c1, c0 = -4 * c2 * math.cos(w0), c2 * (2 * math.cos(w0) ** 2 + 1)
    w = inversion_omega(0.3)
    exp = 10.0 / (c0 + c1 + c2) * (c0 + c1 * math.cos(w) + c2 * math.cos(2 * w))
    assert energy("inversion", inversion_positions(0.3), [w0, 10.0], 4) == pytest.approx(exp, rel=1e-7)


def test_two_body_and_harmonic_angle_known_answers():
    pos = np.array([[0, 0, 0], [1.7, 0, 0.0]])
    assert energy("harmonic_bond", pos, [1.2, 3.0], 2) == pytest.approx((1.7 - 1.2) ** 2 * 3.0)
    assert energy("morse_bond", pos, [1.2, 2.0, 1.5], 2) == pytest.approx(2.0 * (1 - math.exp(-1.5 * 0.5)) ** 2)
    pos = np.array([[0, 0, 0], [1.0, 0, 0], [0, 2.0, 0]])
    assert energy("harmonic_angle", pos, [109.5, 0.02], 3) == pytest.approx((90.0 - 109.5) ** 2 * 0.02)


@pytest.mark.parametrize("kind", list(ob.KINDS))
def test_oracle_gradients_match_total_energy_differences(kind):
    """dE/dx and dE/dtril (Cartesian positions fixed) of the oracle against central
    differences of the total energy in positions and in tril, with image shifts."""
    rng = np.random.default_rng(1)
    _, order = ob.KINDS[kind]
    T, N, E = 2, 12, 10
    tril = np.array([[7.0, 0.8, 6.5, -0.6, 0.9, 7.5]])
    pos = rng.uniform(0, 6, (N, 3))
    edges = np.array([rng.choice(N, order, replace=False) for _ in range(E)])
    shifts = rng.integers(-1, 2, (E, order - 1, 3))
    npar = {"harmonic_bond": 2, "morse_bond": 3, "harmonic_angle": 2, "cosine_angle": 3, "dihedral": 3,
            "inversion": 2}[kind]
    table = rng.uniform(0.5, 2.0, (T**order, npar))
    if kind == "cosine_angle":
        table[:, 2] = math.radians(5)
    species = rng.integers(0, T, N)
    sysi = np.zeros(N, int)
    e, g, gt = ob.bonded(kind, pos, sysi, species, tril, table, T, edges, shifts)
    h = 1e-6
    for i in range(N):
        for a in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[i, a] += h
            p2[i, a] -= h
            fd = (ob.bonded(kind, p1, sysi, species, tril, table, T, edges, shifts)[0][0]
                  - ob.bonded(kind, p2, sysi, species, tril, table, T, edges, shifts)[0][0]) / (2 * h)
            assert fd == pytest.approx(g[i, a], rel=1e-5, abs=1e-6 * max(1.0, np.abs(g).max()))
    for k in range(6):
        t1, t2 = tril.copy(), tril.copy()
        t1[0, k] += h
        t2[0, k] -= h
        fd = (ob.bonded(kind, pos, sysi, species, t1, table, T, edges, shifts)[0][0]
              - ob.bonded(kind, pos, sysi, species, t2, table, T, edges, shifts)[0][0]) / (2 * h)
        assert fd == pytest.approx(gt[0, k], rel=1e-5, abs=1e-6 * max(1.0, np.abs(gt).max()))


def test_morse_known_answers_with_species_pairs():
    """test/potential/classical/test_morse.py:35-133: two species with asymmetric-looking but
    symmetric pair tables, the (A, B) pair evaluated: zero at r0, the dissociation limit D,
    compression above extension, the closed form at r = 1, zero gradient at r0, within 5 % of
    the harmonic bond with k = D alpha^2 near r0; MorseBondParameters.from_harmonic."""
    from kups_gb300.bonded import MorseBondParameters

    r0 = np.array([[1.5, 1.2], [1.2, 1.8]])
    D = np.array([[2.0, 1.5], [1.5, 2.5]])
    alpha = np.array([[2.0, 1.8], [1.8, 2.2]])
    table = np.stack([r0, D, alpha], -1).reshape(4, 3)
    species = np.array([0, 1])

    def morse(r, kind="morse_bond", tab=table):
        pos = np.array([[0.0, 0, 0], [r, 0, 0]])
        e, g, _ = ob.bonded(kind, pos, np.zeros(2, int), species, BOX * 10, tab, 2, np.array([[0, 1]]),
                            np.zeros((1, 1, 3)))
        return e[0], g

    assert morse(1.2)[0] == pytest.approx(0.0, abs=1e-10)
    assert morse(1.5)[0] > 0
    assert morse(100.0)[0] == pytest.approx(1.5, rel=1e-6)
    assert morse(1.2 - 0.3)[0] > morse(1.2 + 0.3)[0]
    assert morse(1.0)[0] == pytest.approx(1.5 * (1 - math.exp(-1.8 * (1.0 - 1.2))) ** 2, rel=1e-6)
    np.testing.assert_allclose(morse(1.2)[1], 0.0, atol=1e-6)
    assert np.linalg.norm(morse(1.5)[1]) > 1e-6
    harmonic = np.stack([r0, D * alpha**2], -1).reshape(4, 2)
    assert morse(1.21)[0] == pytest.approx(morse(1.21, "harmonic_bond", harmonic)[0], rel=0.05)
    k = np.array([[100.0, 80.0], [80.0, 120.0]])
    p = MorseBondParameters.from_harmonic(("A", "B"), np.array([[1.0, 1.2], [1.2, 1.5]]), k, D)
    np.testing.assert_allclose(p.alpha, np.sqrt(k / D))
    np.testing.assert_allclose(p.D, D)


def _energy_grad(kind, pos, row, order, edges=None, system=None, boxes=None):
    T = 1
    table = np.asarray(row, np.float64).reshape(1, -1)
    edges = np.arange(order)[None] if edges is None else np.asarray(edges)
    system = np.zeros(len(pos), int) if system is None else np.asarray(system)
    boxes = BOX if boxes is None else boxes
    return ob.bonded(kind, pos, system, np.zeros(len(pos), int), boxes, table, T, edges,
                     np.zeros((len(edges), order - 1, 3)))


def test_remaining_cosine_angle_and_inversion_cases():
    """test/potential/classical/test_cosine_angle.py:61-110 (zero gradient at theta0 for 90,
    120, 180 degrees, positive energy and non-zero gradient away from it, zero force constant)
    and test_inversion.py:140-205 (zero force constant, the three cyclic orderings of one
    centre, two systems in one call)."""
    def angle_pos(t):
        return np.array([[0, 0, 0], [1.0, 0, 0], [math.cos(t), math.sin(t), 0]])

    for deg, away in ((90, 60), (120, 90), (180, 90)):
        t0 = math.radians(deg)
        e, g, _ = _energy_grad("cosine_angle", angle_pos(t0), [t0, 3.0, math.radians(5)], 3)
        assert e[0] == pytest.approx(0.0, abs=1e-10)
        np.testing.assert_allclose(g, 0.0, atol=1e-6)
        e, g, _ = _energy_grad("cosine_angle", angle_pos(math.radians(away)), [t0, 3.0, math.radians(5)], 3)
        assert e[0] > 0 and np.linalg.norm(g) > 1e-6
    e, _, _ = _energy_grad("cosine_angle", angle_pos(0.7), [math.pi / 2, 0.0, math.radians(5)], 3)
    assert e[0] == pytest.approx(0.0, abs=1e-10)

    e, _, _ = _energy_grad("inversion", inversion_positions(0.5), [0.0, 0.0], 4)
    assert e[0] == pytest.approx(0.0, abs=1e-10)
    e, _, _ = _energy_grad("inversion", inversion_positions(0.2), [0.0, 10.0], 4,
                           edges=[[0, 1, 2, 3], [0, 2, 3, 1], [0, 3, 1, 2]])
    assert e[0] > 0 and np.isfinite(e[0])
    pos = np.concatenate([inversion_positions(0.0), inversion_positions(0.5)])
    e, _, _ = _energy_grad("inversion", pos, [0.0, 10.0], 4, edges=[[0, 1, 2, 3], [4, 5, 6, 7]],
                           system=[0] * 4 + [1] * 4, boxes=np.repeat(BOX, 2, 0))
    assert e[0] == pytest.approx(0.0, abs=1e-10) and e[1] > 0


def test_harmonic_species_tuple_known_answers():
    """test/potential/test_harmonic.py:70-345: species-indexed tables (the row of an edge is
    its atoms' species in edge order), angles at atom 0, several edges and systems."""
    x0 = np.array([[1.5, 1.2], [1.2, 1.8]])
    kb = np.array([[100.0, 80.0], [80.0, 120.0]])
    bond = np.stack([x0, kb], -1).reshape(4, 2)
    z = np.zeros

    def bonds(pos, species, edges, system=None, boxes=None):
        system = z(len(pos), int) if system is None else np.asarray(system)
        boxes = np.array([[10.0, 0, 10.0, 0, 0, 10.0]]) if boxes is None else boxes
        return ob.bonded("harmonic_bond", np.asarray(pos, float), system, np.asarray(species), boxes, bond, 2,
                         np.asarray(edges), z((len(edges), 1, 3)))[0]

    assert bonds([[0, 0, 0], [1.0, 0, 0]], [0, 1], [[0, 1]])[0] == pytest.approx((1.0 - 1.2) ** 2 * 80.0)
    assert bonds([[0, 0, 0], [1.2, 0, 0]], [0, 1], [[0, 1]])[0] == pytest.approx(0.0, abs=1e-10)
    assert bonds([[0, 0, 0], [1.5, 0, 0]], [0, 0], [[0, 1]])[0] == pytest.approx(0.0, abs=1e-10)
    e = bonds([[0, 0, 0], [1.0, 0, 0], [2.5, 0, 0]], [0, 1, 0], [[0, 1], [1, 2]])[0]
    assert e == pytest.approx((1.0 - 1.2) ** 2 * 80.0 + (1.5 - 1.2) ** 2 * 80.0)
    e = bonds([[0, 0, 0], [1.0, 0, 0], [0, 0, 0], [2.0, 0, 0]], [0, 1, 0, 1], [[0, 1], [2, 3]], [0, 0, 1, 1],
              np.tile([10.0, 0, 10.0, 0, 0, 10.0], (2, 1)))
    np.testing.assert_allclose(e, [(1.0 - 1.2) ** 2 * 80.0, (2.0 - 1.2) ** 2 * 80.0])

    theta0 = np.array([[[120.0, 90.0], [90.0, 120.0]], [[90.0, 90.0], [120.0, 90.0]]])
    ka = np.array([[[10.0, 8.0], [12.0, 10.0]], [[8.0, 12.0], [10.0, 8.0]]])
    angle = np.stack([theta0, ka], -1).reshape(8, 2)

    def angles(pos, edges, system, boxes, tab=angle):
        sp = np.tile([0, 1, 0], len(pos) // 3)
        return ob.bonded("harmonic_angle", np.asarray(pos, float), np.asarray(system), sp, boxes, tab, 2,
                         np.asarray(edges), z((len(edges), 2, 3)))[0]

    box1 = np.array([[10.0, 0, 10.0, 0, 0, 10.0]])
    base = [[1.0, 0, 0], [0, 0, 0], [1.0, 1.0, 0]]  # 90 degrees at atom 0, table entry (A, B, A) = 90
    assert angles(base, [[0, 1, 2]], [0, 0, 0], box1)[0] == pytest.approx(0.0, abs=1e-6)
    zero_k = np.stack([theta0, np.zeros_like(ka)], -1).reshape(8, 2)
    assert angles(base, [[0, 1, 2]], [0, 0, 0], box1, zero_k)[0] == pytest.approx(0.0, abs=1e-10)
    e = angles([[0, 0, 0], [1.0, 0, 0], [2.0, 0, 0]], [[0, 1, 2]], [0, 0, 0], box1)[0]
    assert e == pytest.approx((180.0 - 90.0) ** 2 * 12.0, rel=1e-5)  # k[A, B, A] = 12
    e = angles(base + [[1.0, 0, 0], [0, 0, 0], [1.5, 0.866, 0]], [[0, 1, 2], [3, 4, 5]], [0, 0, 0, 1, 1, 1],
               np.repeat(box1, 2, 0))
    theta = math.degrees(math.acos(np.dot([-1.0, 0, 0], [0.5, 0.866, 0]) / np.linalg.norm([0.5, 0.866, 0])))
    np.testing.assert_allclose(e, [0.0, (theta - 90.0) ** 2 * 12.0], rtol=1e-6, atol=1e-9)
