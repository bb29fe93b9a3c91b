"""Replay of free-running GPU GCMC steps against the float64 oracle of the Monte Carlo step.

The kernel's per-step record (``kups_gcmc_trace``) is checked step by step for every system:

* the move kind of each step (shared by all systems) and the molecule it picks;
* the proposed positions of all five kinds (translate, rotate, reinsert, insert, delete),
  regenerated by the oracle from the same Philox draws in float64: within 2e-4 A;
* ln acc against the oracle's muVT ratio (src/kups/mcmc/probability.py:116-225) of the
  device's energy change: within 1e-10 absolute + 1e-12 relative;
* the accept decision: bit-exact (ln acc > ln u, u regenerated by the oracle);
* each move's step width against the oracle's acceptance_target_schedule
  (src/kups/core/parameter_scheduler.py:161-208) fed the same decisions: 1e-5 relative;
* on a sample of steps, the energy change against E_oracle(after) - E_oracle(before):
  2e-5 eV + 2e-5 relative.
"""

import numpy as np
import pytest

from oracle import mcmc as om

from test_gpu_gcmc import oracle_energy, random_molecule, small_setup, wrapped

pytestmark = pytest.mark.gpu


def _replay(rc, seed, n_steps, energy_every, block_threads=0):
    from kups_gb300 import gcmc
    from oracle import unitcell as ouc

    S = 3
    setup = small_setup(n_sys=S, rc=rc)
    setup.log_activity = np.full(S, -6.0)
    setup.max_mol = 48  # room for every insertion the run may accept (a V ~ 4 molecules)
    L = ouc.lattice_from_tril(setup.tril[0])
    rng = np.random.default_rng(seed)
    apm = len(setup.motif_charges)
    guests = [np.concatenate([wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
                              for _ in range(4)]) for _ in range(S)]
    mc = gcmc.GCMC(setup, seed=seed)
    mc.block_threads = block_threads
    mc.set_guests(guests)
    # the device holds float32 positions: the oracle state starts from those
    state = [g.reshape(-1, apm, 3).astype(np.float32).astype(np.float64) for g in guests]
    tr = mc.run_traced(n_steps)
    vol = abs(np.prod(setup.tril[0, [0, 2, 5]]))
    width_max = mc.width_max.cpu().numpy()
    sched = [[om.AcceptanceScheduler(0.1, upper=(float(width_max[s, k]) if width_max[s, k] > 0 else None))
              for k in range(4)] for s in range(S)]
    kinds_seen = set()
    n_energy = 0
    for t in range(n_steps):
        ctr = t  # the sampler starts at step 0
        kind = om.move_kind(seed, ctr, mc.move_cum)
        for s in range(S):
            r = tr[t, s]
            assert r["kind"] == kind, (t, s)
            n_old = len(state[s])
            assert r["n_mol"] == n_old, (t, s)
            sk = 3 if kind >= 3 else kind
            np.testing.assert_allclose(r["width"], sched[s][sk].value, rtol=1e-5, err_msg=f"width {t} {s}")
            mol, new, has_old = om.propose(seed, ctr, s, kind, n_old, state[s], setup.motif_positions,
                                           float(r["width"]), setup.tril[s])
            assert r["mol"] == mol and bool(r["has_old"]) == has_old, (t, s, r["mol"], mol)
            assert bool(r["has_new"]) == (new is not None), (t, s)
            dev_new = r["new_pos"][:apm, :3].astype(np.float64)
            if new is not None:
                d = (dev_new - new) @ np.linalg.inv(L)
                d = (d - np.round(d)) @ L  # either side of a face is the same position
                assert np.abs(d).max() < 2e-4, (t, s, kind, np.abs(d).max())
            n_new = n_old + (1 if kind == 3 else -1 if (kind == 4 and has_old) else 0)
            exp_lp = om.gcmc_log_acceptance(r["de"], setup.temperature[s], setup.log_activity[s], vol, n_old, n_new)
            assert abs(r["log_p"] - exp_lp) <= 1e-10 + 1e-12 * abs(exp_lp), (t, s, r["log_p"], exp_lp)
            lu = om.log_uniform(seed, ctr, s)
            assert abs(r["log_u"] - lu) <= 1e-13, (t, s)
            if abs(r["log_p"] - lu) > 1e-9:
                assert bool(r["accept"]) == (r["log_p"] > lu), (t, s, r["log_p"], lu)
            if energy_every and t % energy_every == 0 and s == 0 and (has_old or new is not None):
                before = state[s].reshape(-1, 3)
                if kind == 3:
                    after = np.concatenate([before, dev_new])
                elif kind == 4:
                    after = np.delete(state[s], mol, 0).reshape(-1, 3)
                else:
                    a = state[s].copy()
                    a[mol] = dev_new
                    after = a.reshape(-1, 3)
                exp = oracle_energy(setup, after) - oracle_energy(setup, before)
                assert abs(r["de"] - exp) <= 2e-5 + 2e-5 * abs(exp), (t, kind, r["de"], exp)
                n_energy += 1
            # apply the decision as the device did (deletion moves the last molecule into the slot)
            # a deletion from an empty system changes nothing (ln acc = 0 accepts it, as the
            # reference accepts a null patch)
            if r["accept"] and (has_old or new is not None):
                if kind == 3:
                    state[s] = np.concatenate([state[s], dev_new[None]])
                elif kind == 4:
                    st = state[s]
                    st[mol] = st[-1]
                    state[s] = st[:-1]
                else:
                    state[s][mol] = dev_new
            sched[s][sk](bool(r["accept"]))
            kinds_seen.add((kind, int(r["accept"])))
    # the device's final state agrees with the replayed one
    dev = mc.guest_positions()
    for s in range(S):
        np.testing.assert_allclose(dev[s], state[s].reshape(-1, 3), atol=1e-6)
        np.testing.assert_allclose(mc.width.cpu().numpy()[s], [sched[s][k].value for k in range(4)], rtol=1e-5)
    return kinds_seen, n_energy, mc


@pytest.mark.parametrize("rc", [5.0, 7.0])  # minimum image / 3 x 3 x 3 image offsets
def test_free_running_steps_replay_exactly(rc):
    kinds_seen, n_energy, mc = _replay(rc, seed=17 if rc == 5.0 else 23, n_steps=1200, energy_every=20)
    # every kind was proposed, and accepted and rejected at least once overall
    assert {k for k, _ in kinds_seen} == {0, 1, 2, 3, 4}
    assert {a for _, a in kinds_seen} == {0, 1}
    assert n_energy >= 25
    # the schedulers moved: 1200 steps give every displacement kind more than 100 moves
    w = mc.width.cpu().numpy()
    assert np.any(np.abs(w[:, :3] - 0.1) > 1e-3)


@pytest.mark.parametrize("threads", [64, 256])
def test_replay_holds_for_every_launch_shape(threads):
    """The autotuner's other CTA sizes run the same chain (600 steps, minimum image)."""
    kinds_seen, _, _ = _replay(5.0, seed=29, n_steps=600, energy_every=0, block_threads=threads)
    assert {k for k, _ in kinds_seen} == {0, 1, 2, 3, 4}
