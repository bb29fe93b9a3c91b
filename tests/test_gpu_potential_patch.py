"""Patched (incremental) potential calls against full recomputation.

``Potential.__call__(state, patch)`` (src/kups/core/potential.py:142-198) with a patch that moves
k particles: E_cached - E(removed edges) + E(added edges) of ``neighborlist_changes``, plus the
Ewald S(k) update, equals the energy of a full call on the moved state.  Bars: 1e-6 eV absolute
for float64 Lennard-Jones (the reference's own bar, test/potential/test_potential_update.py:600-645);
LJ + Ewald 1e-6 relative (float32 reciprocal phases); the float32 LJ pair path 1e-5 relative.
"""

import numpy as np
import pytest
import torch

from test_gpu_core import random_triclinic_batch

pytestmark = pytest.mark.gpu


def cuda(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("seed", [0, 1])
def test_lennard_jones_patch_equals_full(seed, fp32):
    from kups_gb300.potential import LennardJonesParameters, LennardJonesPotential, LJParticles, LJState, ParticlePatch

    pos, sysi, tril, cut, excl, _ = random_triclinic_batch(seed, n_sys=4)
    rng = np.random.default_rng(seed + 9)
    sp = rng.integers(0, 2, len(pos))
    sig = np.array([[1.0, 1.15], [1.15, 1.3]])
    eps = np.array([[0.01, 0.014], [0.014, 0.02]])
    prm = LennardJonesParameters(("A", "B"), torch.as_tensor(sig), torch.as_tensor(eps), torch.as_tensor(cut))
    state = LJState(LJParticles(cuda(pos), cuda(sp, torch.int32), cuda(sysi, torch.int32),
                                exclusion=cuda(excl, torch.int32)), cuda(tril), prm)
    pot = LennardJonesPotential(pair_fp32=fp32)
    full_old = pot(state)
    for trial in range(3):
        k = int(rng.integers(1, 8))
        idx = rng.choice(len(pos), k, replace=False)
        new = pos[idx] + rng.normal(0, 0.8, (k, 3))
        patch = ParticlePatch(cuda(idx, torch.int32), cuda(new))
        got = pot(state, patch, cache=full_old.cache).total_energies.cpu().numpy()
        moved = pos.copy()
        moved[idx] = new
        st2 = LJState(LJParticles(cuda(moved), cuda(sp, torch.int32), cuda(sysi, torch.int32),
                                  exclusion=cuda(excl, torch.int32)), cuda(tril), prm)
        exp = pot(st2).total_energies.cpu().numpy()
        if fp32:
            np.testing.assert_allclose(got, exp, rtol=1e-5, atol=1e-5 * np.abs(exp).max())
        else:
            # the reference's bar is atol 1e-6 (test_potential_update.py); random placements overlap, so
            # energies reach 1e13 where float64 itself resolves only 2e-3: the bar is taken relative there
            np.testing.assert_allclose(got, exp, rtol=1e-13, atol=1e-6)


@pytest.mark.parametrize("rigid", [True, False])
def test_lj_ewald_patch_equals_full(rigid):
    from kups_gb300.ewald import EwaldParameters, EwaldParticles, LJEwaldPotential
    from kups_gb300.potential import ParticlePatch
    from oracle import ewald as oew
    from oracle import unitcell as ouc

    rng = np.random.default_rng(3)
    S, per = 2, 3
    pos, q, sysi, trils, excl = [], [], [], [], []
    for s in range(S):
        L = ouc.lattice_from_lengths_angles(rng.uniform(14, 17, 3), rng.uniform(85, 95, 3))
        m = 20
        c = rng.uniform(-0.5, 0.5, (m, 3)) @ L
        d = rng.normal(0, 1, (m, per, 3))
        d *= 1.1 / np.linalg.norm(d, axis=-1, keepdims=True)
        d[:, 0] = 0.0
        pos.append((c[:, None] + d).reshape(-1, 3))
        qq = np.tile([0.8, -0.4, -0.4], m)
        q.append(qq)
        sysi += [s] * (m * per)
        excl += list(len(excl) // per + np.arange(m * per) // per)
        trils.append(ouc.tril_from_lattice(L))
    pos, q, sysi, tril = np.concatenate(pos), np.concatenate(q), np.array(sysi), np.stack(trils)
    excl = np.arange(len(pos)) // per
    sp = np.tile([0, 1, 1], len(pos) // per)
    n = len(pos)
    # intramolecular pairs, both directions, minimum-image shifts
    xe = np.array([(a, b) for g in range(n // per) for a in range(g * per, g * per + per)
                   for b in range(g * per, g * per + per) if a != b])
    f = np.stack([pos[i] @ np.linalg.inv(ouc.lattice_from_tril(tril[sysi[i]])) for i in range(n)])
    xs = np.round(f[xe[:, 0]] - f[xe[:, 1]]).astype(np.int32)
    kn = np.stack([oew.kvecs_cube(4)] * S).astype(np.int32)
    prm = EwaldParameters(torch.tensor([0.32, 0.3]), torch.tensor([6.5, 7.0]), torch.as_tensor(kn))
    pot = LJEwaldPotential(prm, np.array([[2.8, 3.0], [3.0, 3.1]]), np.array([[0.004, 0.005], [0.005, 0.006]]),
                           np.array([6.0, 6.5]), exclusion_edges=(cuda(xe, torch.int32), cuda(xs, torch.int32)))
    parts = lambda p: EwaldParticles(cuda(p), cuda(q), cuda(sysi, torch.int32), cuda(sp, torch.int32),
                                     cuda(excl, torch.int32))
    old = pot(parts(pos), cuda(tril))
    cache = old.cache
    cur = pos.copy()
    for trial in range(4):
        if rigid:  # whole molecules translated
            g = rng.choice(n // per, 2, replace=False)
            idx = np.concatenate([np.arange(x * per, x * per + per) for x in g])
            new = cur[idx] + np.repeat(rng.normal(0, 1.5, (2, 3)), per, 0)
        else:  # single atoms displaced (the intramolecular correction changes)
            idx = rng.choice(n, 3, replace=False)
            new = cur[idx] + rng.normal(0, 0.2, (3, 3))
        out = pot(parts(cur), cuda(tril), ParticlePatch(cuda(idx, torch.int32), cuda(new)), cache=cache)
        cur = cur.copy()
        cur[idx] = new
        full = pot(parts(cur), cuda(tril))
        got, exp = out.total_energies.cpu().numpy(), full.total_energies.cpu().numpy()
        np.testing.assert_allclose(got, exp, rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(out.cache.structure_factor.cpu().numpy(), full.cache.structure_factor.cpu().numpy(),
                                   atol=2e-6 * float(full.cache.structure_factor.abs().max()))
        cache = out.cache  # accept and continue from the patched cache
