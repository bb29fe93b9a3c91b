"""kups_bonded_edges against the float64 oracle: energies (rtol 1e-10), dE/dx and dE/dtril
(relative 1e-6 of the largest component: the oracle differentiates by central differences)
for every kind, over batched triclinic systems with image shifts, several species and
terms summed into one set of buffers; the reference's known answers through the GPU."""

import math

import numpy as np
import pytest
import torch

from oracle import bonded as ob

pytestmark = pytest.mark.gpu

NPAR = {"harmonic_bond": 2, "morse_bond": 3, "harmonic_angle": 2, "cosine_angle": 3, "dihedral": 3, "inversion": 2}


def params_object(kind, table, T, order):
    from kups_gb300 import bonded

    t = table.reshape((T,) * order + (NPAR[kind],))
    labels = tuple(f"t{i}" for i in range(T))
    if kind == "harmonic_bond":
        return bonded.HarmonicBondParameters(labels, t[..., 0], t[..., 1])
    if kind == "morse_bond":
        return bonded.MorseBondParameters(labels, t[..., 0], t[..., 1], t[..., 2])
    if kind == "harmonic_angle":
        return bonded.HarmonicAngleParameters(labels, t[..., 0], t[..., 1])
    if kind == "cosine_angle":
        return bonded.CosineAngleParameters(labels, t[..., 0], t[..., 1], float(t[..., 2].flat[0]))
    if kind == "dihedral":
        return bonded.DihedralParameters(labels, t[..., 0], t[..., 1], t[..., 2])
    return bonded.InversionParameters(labels, t[..., 0], t[..., 1])


def random_case(kind, rng, S=3, N=40, E=300, T=3):
    _, order = ob.KINDS[kind]
    tril = np.array([[9.0 + s, 0.7 * s, 8.5, -0.5, 0.6, 9.5 - s] for s in range(S)])
    system = np.repeat(np.arange(S), N)
    pos = rng.uniform(0, 8, (S * N, 3))
    edges = []
    for _ in range(E):
        s = rng.integers(S)
        edges.append(s * N + rng.choice(N, order, replace=False))
    edges = np.array(edges)
    shifts = rng.integers(-1, 2, (E, order - 1, 3))
    table = rng.uniform(0.5, 2.0, (T**order, NPAR[kind]))
    if kind == "harmonic_angle":
        table[:, 0] = rng.uniform(80, 130, T**order)
    if kind == "cosine_angle":
        table[:, 0] = np.where(rng.random(T**order) < 0.3, np.pi, rng.uniform(1.6, 2.3, T**order))
        table[:, 2] = math.radians(5)
    if kind == "dihedral":
        table[:, 1] = rng.integers(1, 7, T**order)
        table[:, 2] = rng.choice([0.0, np.pi / 3, np.pi / 2, np.pi], T**order)
    if kind == "inversion":
        table[:, 0] = np.where(rng.random(T**order) < 0.5, 0.0, rng.uniform(0.2, 0.8, T**order))
    species = rng.integers(0, T, S * N)
    return pos, system, species, tril, edges, shifts, table, T, order


@pytest.mark.parametrize("kind", list(ob.KINDS))
def test_bonded_kernel_matches_oracle(kind):
    from kups_gb300 import bonded

    rng = np.random.default_rng(ob.KINDS[kind][0] + 7)
    pos, system, species, tril, edges, shifts, table, T, order = random_case(kind, rng)
    term = bonded.BondedTerm(params_object(kind, table, T, order), edges, shifts)
    e, g, gt = (x.cpu().numpy() for x in bonded.evaluate([term], pos, system, species, tril))
    er, gr, gtr = ob.bonded(kind, pos, system, species, tril, table, T, edges, shifts)
    np.testing.assert_allclose(e, er, rtol=1e-10, atol=1e-12 * np.abs(er).max())
    np.testing.assert_allclose(g, gr, rtol=0, atol=1e-6 * np.abs(gr).max())
    np.testing.assert_allclose(gt, gtr, rtol=0, atol=1e-6 * np.abs(gtr).max())


@pytest.mark.parametrize("kind", list(ob.KINDS))
def test_bonded_fp32_mode_within_float32_tolerance(kind):
    """fp32 != 0: the per-edge arithmetic in float32, so energies to 2e-5 of the largest
    per-system energy (a few hundred edges of float32 rounding each) and gradients to 2e-4 of
    the largest component (angles near 0 or pi amplify the rounding of the cosine)."""
    from kups_gb300 import bonded

    rng = np.random.default_rng(ob.KINDS[kind][0] + 7)
    pos, system, species, tril, edges, shifts, table, T, order = random_case(kind, rng)
    term = bonded.BondedTerm(params_object(kind, table, T, order), edges, shifts, fp32=True)
    e, g, gt = (x.cpu().numpy() for x in bonded.evaluate([term], pos, system, species, tril))
    er, gr, gtr = ob.bonded(kind, pos, system, species, tril, table, T, edges, shifts)
    np.testing.assert_allclose(e, er, rtol=0, atol=2e-5 * np.abs(er).max())
    np.testing.assert_allclose(g, gr, rtol=0, atol=2e-4 * np.abs(gr).max())
    np.testing.assert_allclose(gt, gtr, rtol=0, atol=2e-4 * np.abs(gtr).max())


def test_terms_add_into_one_buffer():
    from kups_gb300 import bonded

    pos, system, species, tril, _, _, _, T, _ = random_case("harmonic_bond", np.random.default_rng(5))
    terms, ref = [], None
    for kind in ("harmonic_bond", "harmonic_angle", "dihedral"):
        order = ob.KINDS[kind][1]
        sub = np.random.default_rng(ob.KINDS[kind][0])
        edges = np.array([sub.choice(40, order, replace=False) for _ in range(50)])
        shifts = sub.integers(-1, 2, (50, order - 1, 3))
        table = sub.uniform(0.5, 2.0, (T**order, NPAR[kind]))
        if kind == "harmonic_angle":
            table[:, 0] = sub.uniform(80, 130, T**order)
        terms.append(bonded.BondedTerm(params_object(kind, table, T, order), edges, shifts))
        r = ob.bonded(kind, pos, system, species, tril, table, T, edges, shifts)
        ref = r if ref is None else tuple(a + b for a, b in zip(ref, r))
    e, g, gt = (x.cpu().numpy() for x in bonded.evaluate(terms, pos, system, species, tril))
    np.testing.assert_allclose(e, ref[0], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(g, ref[1], rtol=0, atol=1e-6 * np.abs(ref[1]).max())
    np.testing.assert_allclose(gt, ref[2], rtol=0, atol=1e-6 * np.abs(ref[2]).max())


def test_known_answers_on_the_gpu():
    """dihedral V = 2, n = 3, phi0 = pi: 0 (trans), 2 (cis), 1 (90 deg)
    (test/potential/classical/test_dihedral.py:157-205)."""
    from kups_gb300 import bonded
    from test_oracle_bonded import dihedral_positions

    pos = np.concatenate([dihedral_positions(p) for p in (np.pi, 0.0, np.pi / 2)])
    system = np.repeat(np.arange(3), 4)
    tril = np.tile([20.0, 0, 20.0, 0, 0, 20.0], (3, 1))
    edges = np.arange(12).reshape(3, 4)
    term = bonded.BondedTerm(bonded.DihedralParameters(("A",), np.full((1,) * 4, 2.0), np.full((1,) * 4, 3.0),
                                                       np.full((1,) * 4, np.pi)), edges)
    e, _, _ = bonded.evaluate([term], pos, system, np.zeros(12, np.int32), tril)
    np.testing.assert_allclose(e.cpu().numpy(), [0.0, 2.0, 1.0], atol=1e-10)


def test_out_of_range_edge_is_reported():
    from kups_gb300 import _lib, bonded

    term = bonded.BondedTerm(bonded.HarmonicBondParameters(("A",), np.ones((1, 1)), np.ones((1, 1))),
                             np.array([[0, 1], [0, 7]]))
    with pytest.raises(_lib.KupsError):
        bonded.evaluate([term], np.zeros((2, 3)) + [[0, 0, 0], [1.0, 0, 0]], np.zeros(2, np.int32),
                        np.zeros(2, np.int32), np.array([[10.0, 0, 10.0, 0, 0, 10.0]]))


def _moved(rng, pos, system, tril, n_changed):
    """Distinct moved atoms, small displacements, new positions wrapped into the cell with
    their lattice offsets (new = unwrapped - n @ L)."""
    from oracle.unitcell import lattice_from_tril, to_fractional

    ch = rng.choice(len(pos), n_changed, replace=False)
    L = lattice_from_tril(tril[system[ch]])
    hop = rng.integers(-1, 2, (n_changed, 3)).astype(float)  # some moves land in a neighbouring cell
    unwrapped = pos[ch] + rng.normal(scale=0.3, size=(n_changed, 3)) + np.einsum("ka,kab->kb", hop, L)
    f = to_fractional(unwrapped, tril[system[ch]])
    n = np.floor(f + 0.5).astype(np.int64)
    new = unwrapped - np.einsum("ka,kab->kb", n.astype(float), L)
    return ch, new, n


@pytest.mark.parametrize("kind", list(ob.KINDS))
@pytest.mark.parametrize("fp32,use_incidence", [(False, True), (True, True), (False, False)])
def test_mc_delta_matches_the_oracle_energy_difference(kind, fp32, use_incidence):
    """kups_bonded_delta (old-graph / new-graph difference over the affected edges,
    graph.py:336-361, 412-450) against the oracle's total energies before and after the move,
    with wrapped moves rewriting the edge shifts; relative 1e-9 (float64 per-edge arithmetic)
    or 2e-5 (float32) of the largest total energy."""
    from kups_gb300 import bonded

    rng = np.random.default_rng(ob.KINDS[kind][0] + 31)
    pos, system, species, tril, edges, shifts, table, T, order = random_case(kind, rng)
    ch, new, n = _moved(rng, pos, system, tril, 25)
    term = bonded.BondedTerm(params_object(kind, table, T, order), edges, shifts, fp32=fp32)
    d = bonded.delta_energy([term], pos, system, species, tril, ch, new, n, use_incidence).cpu().numpy()
    img = np.zeros((len(pos), 3), np.int64)
    img[ch] = n
    pos_new = pos.copy()
    pos_new[ch] = new
    shifts_new = shifts + img[edges[:, 1:]] - img[edges[:, :1]]
    e0 = ob.bonded(kind, pos, system, species, tril, table, T, edges, shifts)[0]
    e1 = ob.bonded(kind, pos_new, system, species, tril, table, T, edges, shifts_new)[0]
    tol = (2e-5 if fp32 else 1e-9) * np.abs(e0).max()
    np.testing.assert_allclose(d, e1 - e0, rtol=0, atol=tol)
    assert np.any(n != 0)  # some moves wrapped


def test_mc_delta_of_null_and_lattice_moves_is_zero():
    from oracle.unitcell import lattice_from_tril

    from kups_gb300 import bonded

    rng = np.random.default_rng(2)
    pos, system, species, tril, edges, shifts, table, T, order = random_case("dihedral", rng)
    term = bonded.BondedTerm(params_object("dihedral", table, T, order), edges, shifts)
    ch = rng.choice(len(pos), 30, replace=False)
    d = bonded.delta_energy([term], pos, system, species, tril, ch, pos[ch]).cpu().numpy()
    assert np.abs(d).max() < 1e-12
    n = rng.integers(-2, 3, (30, 3))
    L = lattice_from_tril(tril[system[ch]])
    moved = pos[ch] - np.einsum("ka,kab->kb", n.astype(float), L)  # the same atoms, other images
    d = bonded.delta_energy([term], pos, system, species, tril, ch, moved, n).cpu().numpy()
    e0 = ob.bonded("dihedral", pos, system, species, tril, table, T, edges, shifts)[0]
    assert np.abs(d).max() < 1e-9 * np.abs(e0).max()


def test_mc_delta_reports_a_bad_index():
    from kups_gb300 import _lib, bonded

    term = bonded.BondedTerm(bonded.HarmonicBondParameters(("A",), np.ones((1, 1)), np.ones((1, 1))),
                             np.array([[0, 1]]))
    with pytest.raises(_lib.KupsError):
        bonded.delta_energy([term], np.zeros((2, 3)) + [[0, 0, 0], [1.0, 0, 0]], np.zeros(2, np.int32),
                            np.zeros(2, np.int32), np.array([[10.0, 0, 10.0, 0, 0, 10.0]]), [5], [[0.0, 0, 0]])
