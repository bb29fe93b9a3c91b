"""kups_virial_stress against the float64 oracle: atomic, molecular (RASPA convention) and
lattice-gradient stress, kinetic energy and pressure over batched triclinic systems with
molecules straddling the cell faces (relative 1e-11 of the largest component: the sums run
in a different order), in system-sorted and shuffled particle order; the reference's known
answers through the GPU; bad indices reported."""

import numpy as np
import pytest
import torch

from oracle import observables as ob
from oracle.md import kinetic_energy
from oracle.unitcell import lattice_from_tril, wrap

pytestmark = pytest.mark.gpu


def batched_case(seed, S=5, n_mol=(40, 300), size=3, shuffle=False):
    rng = np.random.default_rng(seed)
    trils, pos, sysi, grp = [], [], [], []
    g0 = 0
    for s in range(S):
        t = np.array([10.0 + s, 0.6 * s, 9.0 + 0.5 * s, -0.4, 0.5, 11.0 - 0.3 * s])
        m = int(rng.integers(*n_mol))
        L = lattice_from_tril(t)
        c = rng.uniform(-0.5, 0.5, (m, 3)) @ L
        p = (c[:, None, :] + rng.normal(scale=0.7, size=(m, size, 3))).reshape(-1, 3)
        trils.append(t)
        pos.append(wrap(p, t[None]))
        sysi.append(np.full(m * size, s))
        grp.append(g0 + np.repeat(np.arange(m), size))
        g0 += m
    tril, pos, sysi, grp = np.array(trils), np.concatenate(pos), np.concatenate(sysi), np.concatenate(grp)
    n = len(pos)
    grad = rng.normal(size=(n, 3))
    dtril = rng.normal(size=(S, 6))
    mom = rng.normal(size=(n, 3))
    mass = rng.uniform(1.0, 40.0, n)
    if shuffle:
        o = rng.permutation(n)
        pos, sysi, grp, grad, mom, mass = pos[o], sysi[o], grp[o], grad[o], mom[o], mass[o]
    return pos, grad, sysi, grp, g0, tril, dtril, mom, mass


def close(a, b, rel=1e-11):
    b = np.asarray(b)
    np.testing.assert_allclose(np.asarray(a), b, rtol=0, atol=rel * max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("shuffle", [False, True])
def test_virial_observables_match_the_oracle(shuffle):
    from kups_gb300 import observables

    pos, grad, sysi, grp, G, tril, dtril, mom, mass = batched_case(11 + shuffle, shuffle=shuffle)
    out = observables.virial_observables(pos, grad, sysi, tril, dtril, group=grp, n_groups=G, momenta=mom,
                                         masses=mass, molecular=True)
    out = {k: v.cpu().numpy() for k, v in out.items()}
    st = ob.virial_stress(pos, grad, sysi, tril, dtril)
    ke = kinetic_energy(mom, mass, sysi, len(tril))
    close(out["stress"], st)
    close(out["molecular_stress"], ob.molecular_virial_stress(pos, grad, sysi, grp, G, tril, dtril))
    close(out["lattice_stress"], ob.lattice_stress(tril, dtril))
    close(out["kinetic"], ke)
    close(out["pressure"], ob.instantaneous_pressure(ke, st, tril))


def test_large_batch_without_momenta():
    """1.5e6 atoms in 64 systems, no momenta: pressure = Tr(stress) / 3, the molecular stress of
    single-atom groups is the symmetrised atomic stress (size-independent identities)."""
    from kups_gb300 import observables

    S, per = 64, 24000
    rng = np.random.default_rng(5)
    tril = np.tile([30.0, 1.0, 29.0, -2.0, 0.5, 31.0], (S, 1))
    sysi = np.repeat(np.arange(S), per)
    pos = wrap(rng.uniform(-15, 15, (S * per, 3)), tril[sysi])
    grad = rng.normal(size=(S * per, 3))
    dtril = rng.normal(size=(S, 6))
    out = observables.virial_observables(pos, grad, sysi, tril, dtril, group=np.arange(S * per), molecular=True)
    st = out["stress"].cpu().numpy()
    close(st, ob.virial_stress(pos, grad, sysi, tril, dtril), rel=1e-10)
    close(out["pressure"].cpu().numpy(), np.trace(st, axis1=1, axis2=2) / 3)
    L = lattice_from_tril(tril)
    G = lattice_from_tril(dtril)
    V = np.abs(np.linalg.det(L))[:, None, None]
    LtG = np.swapaxes(L, 1, 2) @ G
    A = -st * V - LtG
    close(out["molecular_stress"].cpu().numpy(), (-0.5 * (A + np.swapaxes(A, 1, 2)) - LtG) / V, rel=1e-9)


def test_known_answers_on_the_gpu():
    """test/observables/test_stress.py:110-160 and the lattice-gradient cases (:75-105)."""
    from kups_gb300 import observables

    r = np.array([[1.0, 0, 0], [0, 1.0, 0]])
    s = observables.stress_via_virial_theorem(r, r, [0, 0], [[2.0, 0, 2.0, 0, 0, 2.0]]).cpu().numpy()[0]
    np.testing.assert_allclose(s, -(np.outer(r[0], r[0]) + np.outer(r[1], r[1])) / 8.0, rtol=1e-12)
    s = observables.stress_via_virial_theorem(np.zeros((1, 3)), np.zeros((1, 3)), [0], [[2.0, 0, 2.0, 0, 0, 2.0]],
                                              [[3.0, 0, 3.0, 0, 0, 3.0]]).cpu().numpy()[0]
    np.testing.assert_allclose(s, -np.eye(3) * 6.0 / 8.0, rtol=1e-12)
    s = observables.stress_via_lattice_vector_gradients([[2.0, 0, 2.0, 0, 0, 2.0]], [[1.0, 3.0, 4.0, 0, 0, 5.0]])
    np.testing.assert_allclose(s.cpu().numpy()[0], -np.array([[1.0, 0, 0], [3.0, 4.0, 0], [0, 0, 5.0]]) / 8.0,
                               rtol=1e-12)
    rr = np.random.default_rng(0).normal(size=(5, 3))
    gg = np.random.default_rng(1).normal(size=(5, 3))
    s = observables.stress_via_virial_theorem(rr, gg, np.zeros(5), [[2.0, 0, 2.0, 0, 0, 2.0]]).cpu().numpy()[0]
    np.testing.assert_allclose(s, -(gg[:, None] * rr[..., None]).sum(0) / 8.0, rtol=1e-12)  # stress.py:77


def test_bad_indices_are_reported():
    from kups_gb300 import _lib, observables

    pos, grad = np.zeros((3, 3)), np.ones((3, 3))
    tril = [[5.0, 0, 5.0, 0, 0, 5.0]]
    with pytest.raises(_lib.KupsError):
        observables.virial_observables(pos, grad, [0, 1, 0], tril)
    with pytest.raises(_lib.KupsError):
        observables.virial_observables(pos, grad, [0, 0, 0], tril, group=[0, 5, 1], n_groups=2, molecular=True)
