"""FusedLennardJonesMD.propagate_host: a state in pinned host memory propagated in runs of whole
systems with the host <-> device copies overlapped, against the device call on the same state.

Bar: bit-exact.  Every system runs in its own CTA, and the random streams are keyed by the
global atom and system index (kups_md_args.atom_base / system_base), so cutting the batch into
runs changes no number.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x)).to("cuda", dtype)


def state_of(W, perm=None, npt=False):
    from kups_gb300 import md, potential

    S = W.n_systems
    perm = np.arange(W.n_atoms) if perm is None else perm
    dt = float(W.time_step[0])
    full = lambda x: cuda(np.full(S, x, np.float64))
    prm = potential.LennardJonesParameters("Ar", torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(cuda(W.positions[perm]), cuda(W.momenta[perm]), cuda(W.masses[perm]),
                           cuda(W.species[perm], torch.int32), cuda(W.system[perm], torch.int32), None)
    systems = md.MDSystems(cuda(W.tril), cuda(W.time_step), cuda(W.temperature), cuda(W.friction),
                           thermostat_time_constant=full(20 * dt), target_pressure=full(0.0),
                           pressure_coupling_time=full(10 * dt), compressibility=full(1e-4 if npt else 0.0),
                           minimum_scale_factor=full(0.9))
    return md.MDState(parts, systems, prm, skin=W.skin)


def to_host(state):
    """The same state with positions and momenta in pinned host memory (static arrays stay)."""
    from dataclasses import replace

    p = state.particles
    pin = lambda t: t.cpu().pin_memory()
    return replace(state, particles=replace(p, positions=pin(p.positions), momenta=pin(p.momenta),
                                            forces=None if p.forces is None else pin(p.forces)))


def assert_same(dev_out, host_out, npt):
    for f in ("positions", "momenta", "forces"):
        np.testing.assert_array_equal(getattr(dev_out.particles, f).cpu().numpy(),
                                      getattr(host_out.particles, f).numpy(), err_msg=f)
    for f in ("potential_energy", "kinetic_energy"):
        np.testing.assert_array_equal(getattr(dev_out.systems, f).cpu().numpy(),
                                      getattr(host_out.systems, f).cpu().numpy(), err_msg=f)
    if npt:
        np.testing.assert_array_equal(dev_out.systems.tril.cpu().numpy(), host_out.systems.tril.cpu().numpy())


@pytest.mark.parametrize("integrator", ["velocity_verlet", "baoab", "csvr", "csvr_npt"])
def test_propagate_host_equals_the_device_call(integrator):
    from kups_gb300 import md, workloads

    W = workloads.batched_uneven_lj(n_systems=24, n_min=64, n_max=500, seed=5)
    npt = integrator == "csvr_npt"
    a = md.FusedLennardJonesMD(integrator, steps_per_call=15)
    b = md.FusedLennardJonesMD(integrator, steps_per_call=15)
    sa = state_of(W, npt=npt)
    sb = to_host(state_of(W, npt=npt))
    for call in range(3):  # later calls resume each run's Verlet lists
        sa = a([3, call], sa)
        sb = b.propagate_host([3, call], sb, chunks=4)
        assert_same(sa, sb, npt)
        assert not sb.particles.positions.is_cuda
    assert len(b._host.bounds) == 4
    assert [r[0] for r in b._host.bounds] == sorted({r[0] for r in b._host.bounds})


def test_propagate_host_of_an_ungrouped_table_runs_one_batch():
    """Atoms not grouped by system: one run, still the device call's result."""
    from kups_gb300 import md, workloads

    W = workloads.batched_uneven_lj(n_systems=10, n_min=64, n_max=300, seed=8)
    perm = np.random.default_rng(0).permutation(W.n_atoms)
    a = md.make_baoab_langevin_step(steps_per_call=10)
    b = md.make_baoab_langevin_step(steps_per_call=10)
    sa = a(5, state_of(W, perm))
    sb = b.propagate_host(5, to_host(state_of(W, perm)), chunks=4)
    assert len(b._host.bounds) == 1
    assert_same(sa, sb, False)


def test_propagate_host_retries_a_run_that_overflows_its_lists():
    from kups_gb300 import md, workloads

    W = workloads.batched_uneven_lj(n_systems=12, n_min=64, n_max=400, seed=9)
    a = md.FusedLennardJonesMD("baoab", 10, neighbor_capacity=256)
    b = md.FusedLennardJonesMD("baoab", 10)
    sa = a(1, state_of(W))
    sb = b.propagate_host(1, to_host(state_of(W)), chunks=3)
    assert_same(sa, sb, False)
    # a run that starts from a capacity far too small overflows, is restored and rerun
    c = md.FusedLennardJonesMD("baoab", 10)
    c._host_run(to_host(state_of(W)), 3)
    for sub in c._host.props:
        sub.neighbor_capacity = 16
    sc = c.propagate_host(1, to_host(state_of(W)), chunks=3)
    assert_same(sa, sc, False)
    assert all(sub.neighbor_capacity > 16 for sub in c._host.props)
