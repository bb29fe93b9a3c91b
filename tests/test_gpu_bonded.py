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
