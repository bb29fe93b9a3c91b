"""CSVR thermostat and CSVR + stochastic cell-rescaling (NPT) integrators of the fused
Lennard-Jones MD kernel against the float64 oracle (md/integrators.py:469-890).

Deterministic parity: at zero target temperature both stochastic terms vanish, so the
whole NPT trajectory (thermostat scale sqrt(exp(-dt / tau_T)), pressure from the pair
virial, cell and position scaling, forces again) is compared step for step with the
oracle.  Limits: tau_T = inf reproduces velocity Verlet bit for bit and zero
compressibility reproduces CSVR bit for bit.  Statistics: the CSVR kinetic energy of an
ideal gas follows the canonical Gamma(N_dof / 2, kT) law.  The Verlet list's validity
under cell scaling is checked by comparing forces after strong compression / expansion
with forces recomputed by the oracle from scratch.
"""

import numpy as np
import pytest
import torch

from oracle import md as omd
from oracle.units import BOLTZMANN_CONSTANT

pytestmark = pytest.mark.gpu

FORCE_RMS_TOL = 1e-5
P_SCALE = 2.6e-4  # argon epsilon / sigma^3 in eV / A^3: the pressure scale of these fluids


def cuda(x, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x)).to("cuda", dtype)


def workload(n_systems=4, n_max=300, seed=5, n_min=64):
    from kups_gb300 import workloads

    return workloads.batched_uneven_lj(n_systems=n_systems, n_min=n_min, n_max=n_max, seed=seed)


def state_of(W, temperature=None, tau_t=None, p0=None, tau_p=None, beta=None, min_scale=0.9):
    from kups_gb300 import md, potential

    S = W.n_systems
    temperature = W.temperature if temperature is None else temperature
    prm = potential.LennardJonesParameters("Ar", torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(cuda(W.positions), cuda(W.momenta), cuda(W.masses), cuda(W.species, torch.int32),
                           cuda(W.system, torch.int32), None)
    full = lambda x: None if x is None else cuda(np.broadcast_to(np.asarray(x, np.float64), (S,)).copy())
    systems = md.MDSystems(cuda(W.tril), cuda(W.time_step), cuda(temperature), cuda(W.friction),
                           thermostat_time_constant=full(tau_t), target_pressure=full(p0),
                           pressure_coupling_time=full(tau_p), compressibility=full(beta),
                           minimum_scale_factor=full(min_scale))
    return md.MDState(parts, systems, prm, skin=W.skin)


def oracle_pressure(W, pos, mom, tril):
    cut = np.full(W.n_systems, W.cutoff)
    _, f, dtr = omd.lj_forces(pos, W.system, W.species, tril, W.sigma, W.epsilon, cut)
    ke = omd.kinetic_energy(mom, W.masses, W.system, W.n_systems)
    return omd.instantaneous_pressure(ke, omd.virial_stress(pos, -f, W.system, tril, dtr), tril), f


def test_csvr_with_infinite_tau_is_velocity_verlet_bit_for_bit():
    from kups_gb300 import md

    W = workload(n_systems=6, n_max=500, seed=3)
    a = md.make_velocity_verlet_step(steps_per_call=25)(7, state_of(W))
    b = md.make_csvr_step(steps_per_call=25)(7, state_of(W, tau_t=np.inf))
    for x, y in ((a.particles.positions, b.particles.positions), (a.particles.momenta, b.particles.momenta)):
        assert torch.equal(x, y)


def test_npt_with_zero_compressibility_is_csvr_bit_for_bit():
    from kups_gb300 import md

    W = workload(n_systems=6, n_max=500, seed=4)
    tau = 50 * W.time_step[0]
    a = md.make_csvr_step(steps_per_call=25)(11, state_of(W, tau_t=tau))
    b = md.make_csvr_npt_step(steps_per_call=25)(11, state_of(W, tau_t=tau, p0=0.0, tau_p=tau, beta=0.0))
    assert torch.equal(a.particles.positions, b.particles.positions)
    assert torch.equal(a.particles.momenta, b.particles.momenta)
    assert torch.equal(b.systems.tril.cpu(), torch.as_tensor(W.tril))


@pytest.mark.parametrize("integrator", ["csvr", "csvr_npt"])
def test_zero_temperature_trajectory_matches_oracle(integrator):
    """kT = 0: alpha = sqrt(exp(-dt / tau_T)) and the barostat is deterministic; 8 steps
    against the oracle (positions 1e-3 A, cell rtol 1e-6, energies and final pressure 1e-4)."""
    from kups_gb300 import md

    W = workload()
    S = W.n_systems
    dt = W.time_step[0]
    tau_t, tau_p = 20 * dt, 10 * dt
    p_init, _ = oracle_pressure(W, W.positions, W.momenta, W.tril)
    beta = 3e-3 * (tau_p / dt) / np.maximum(np.abs(p_init), P_SCALE)  # |d eps| <~ 3e-3 at the first step
    zero = np.zeros(S)
    n_steps = 8
    npt = integrator == "csvr_npt"
    prop = (md.make_csvr_npt_step if npt else md.make_csvr_step)(steps_per_call=n_steps)
    out = prop(0, state_of(W, temperature=zero, tau_t=tau_t, p0=zero, tau_p=tau_p, beta=beta))
    cut = np.full(S, W.cutoff)
    _, f0, _ = omd.lj_forces(W.positions, W.system, W.species, W.tril, W.sigma, W.epsilon, cut)
    rz = np.zeros((n_steps, S))
    pos, mom, f, tril, e, _ = omd.csvr_npt(W.positions, W.momenta, f0, W.masses, W.system, W.species, W.tril,
                                           W.sigma, W.epsilon, cut, W.time_step, zero, np.full(S, tau_t), zero,
                                           np.full(S, tau_p), beta, np.full(S, 0.9), rz, rz, rz, barostat=npt)
    gtril = out.systems.tril.cpu().numpy()
    np.testing.assert_allclose(gtril, tril, rtol=1e-6)
    if npt:
        assert np.all(np.abs(tril[:, 0] / W.tril[:, 0] - 1) > 1e-3)  # the cell did move
    gpos = out.particles.positions.cpu().numpy()
    d = omd._wrap_all(gpos - pos, W.system, tril)
    assert np.abs(d).max() < 1e-3
    np.testing.assert_allclose(out.particles.momenta.cpu().numpy(), mom, atol=1e-3 * np.abs(mom).max())
    np.testing.assert_allclose(out.systems.potential_energy.cpu().numpy(), e[-1], rtol=1e-4)
    p_ref, _ = oracle_pressure(W, pos, mom, tril)
    np.testing.assert_allclose(out.systems.pressure.cpu().numpy(), p_ref, rtol=1e-3,
                               atol=1e-3 * np.abs(p_ref).max())


def test_verlet_list_stays_exact_under_strong_cell_scaling():
    """Targets far above / below the current pressure drive the cells down / up by
    several percent over 120 steps; the kernel's forces at the end equal forces the
    oracle recomputes from scratch at the returned positions and cell."""
    from kups_gb300 import md

    W = workload(n_systems=6, n_max=600, seed=8)
    S = W.n_systems
    dt = W.time_step[0]
    tau_p = 20 * dt
    p_init, _ = oracle_pressure(W, W.positions, W.momenta, W.tril)
    span = 4 * np.maximum(np.abs(p_init), P_SCALE)
    p0 = np.where(np.arange(S) % 2 == 0, p_init + span, p_init - span)
    beta = 2e-3 * (tau_p / dt) / np.abs(p0 - p_init)
    prop = md.make_csvr_npt_step(steps_per_call=120)
    out = prop(5, state_of(W, tau_t=20 * dt, p0=p0, tau_p=tau_p, beta=beta, min_scale=0.99))
    tril = out.systems.tril.cpu().numpy()
    ratio = tril[:, 0] / W.tril[:, 0]
    assert np.all(ratio[0::2] < 0.99) and np.all(ratio[1::2] > 1.01), ratio
    np.testing.assert_allclose(tril[:, 2] / W.tril[:, 2], ratio, rtol=1e-12)
    pos = out.particles.positions.cpu().numpy()
    e, f, _ = omd.lj_forces(pos, W.system, W.species, tril, W.sigma, W.epsilon, np.full(S, W.cutoff))
    gf = out.particles.forces.cpu().numpy()
    rms = np.sqrt(np.mean((gf - f) ** 2)) / np.sqrt(np.mean(f**2))
    assert rms <= FORCE_RMS_TOL, rms
    np.testing.assert_allclose(out.systems.potential_energy.cpu().numpy(), e, rtol=1e-5)


def test_csvr_ideal_gas_kinetic_energy_is_canonical():
    """No forces (epsilon = 0): CSVR alone maps K to alpha^2 K, whose stationary law is
    Gamma(N_dof / 2, kT): mean N_dof kT / 2 and variance N_dof (kT)^2 / 2."""
    from kups_gb300 import md

    W = workload(n_systems=400, n_max=40, seed=9, n_min=20)
    W.epsilon = np.zeros_like(W.epsilon)
    S = W.n_systems
    n_atoms = np.bincount(W.system, minlength=S)
    dof = 3 * n_atoms - 3
    state = state_of(W, tau_t=2 * W.time_step[0])
    prop = md.make_csvr_step()
    packed = md.pack(state)
    _, tke = prop.run_packed(packed, 250, seed=21, trace=True)
    kt = W.temperature * BOLTZMANN_CONSTANT
    x = (tke.cpu().numpy()[50::10] / (0.5 * dof * kt)).reshape(-1)  # K / <K>
    assert abs(x.mean() - 1) < 4 * x.std() / np.sqrt(x.size), x.mean()
    # Var(K) / <K>^2 = 2 / N_dof for a Gamma(N_dof / 2) law
    z = (tke.cpu().numpy()[50::10] / (0.5 * dof * kt) - 1) / np.sqrt(2.0 / dof)
    assert abs(z.reshape(-1).var() - 1) < 0.1, z.var()


def test_npt_cell_and_virial_are_the_same_on_every_run():
    """The barostat reads the pair virial every step; the force pass that forms it takes its atom
    groups in a fixed order, so cells, positions and dE/dtril repeat bit for bit."""
    from kups_gb300 import md

    W = workload(n_systems=8, n_max=900, seed=12)
    dt = W.time_step[0]
    runs = []
    for _ in range(2):
        prop = md.make_csvr_npt_step(steps_per_call=20)
        out = prop(3, state_of(W, tau_t=20 * dt, p0=np.zeros(W.n_systems), tau_p=10 * dt, beta=1e-4))
        runs.append([out.systems.tril.cpu().numpy(), out.particles.positions.cpu().numpy(),
                     out.systems.unitcell_gradients.cpu().numpy()])
    diag = [0, 2, 5]
    assert np.abs(runs[0][0][:, diag] / W.tril[:, diag] - 1).max() > 1e-7  # the cells moved
    for x, y in zip(*runs):
        np.testing.assert_array_equal(x, y)
