"""Molecular-dynamics integrators in float64 (oracle, test infrastructure).

Restates src/kups/md/integrators.py: ``MomentumStep`` (:217-263, B:
p += F dt), ``PositionStep`` with ``MinimumImageConventionFlow`` (:104-211, A:
r += p/m dt then wrap into fractional [-0.5, 0.5)), ``StochasticStep``
(:330-401, O: p = e^{-gamma dt} p + sqrt(kT (1 - e^{-2 gamma dt})) sqrt(m) eta),
``make_velocity_verlet_step`` (:273-318: B(dt/2) A(dt) F B(dt/2)) and
``make_baoab_langevin_step`` (:405-455: B(dt/2) A(dt/2) O(dt) A(dt/2) F B(dt/2));
kinetic energy (src/kups/md/observables.py:17-35) and the Maxwell-Boltzmann
initialisation with centre-of-mass drift removal (application/md/data.py:170-176);
``CSVRStep`` / ``make_csvr_step`` (integrators.py:469-615: momenta scaled by
alpha, alpha^2 = c1 + c2 (R1^2 + R2) + 2 R1 sqrt(c1 c2), then VV) and
``StochasticCellRescalingStep`` / ``make_csvr_npt_step`` (:641-890: CSVR, VV,
cell and positions scaled by mu = clip(exp(d eps / 3)), forces again), with the
virial stress (observables/stress.py:70-82) and the instantaneous pressure
(md/observables.py:38-61) per system.
Forces are -dE/dx from the Lennard-Jones oracle over the reference-exact
neighbour list, rebuilt every step as the reference's MD app does.
"""

from __future__ import annotations

import numpy as np

from .lennard_jones import lj_from_edges
from .neighborlist import neighbor_list
from .unitcell import lattice_from_tril, wrap
from .units import BOLTZMANN_CONSTANT


def lj_forces(pos, system, species, tril, sigma, epsilon, cutoffs):
    e, s = neighbor_list(pos, system, tril, cutoffs)
    energy, grad, dtril = lj_from_edges(pos, system, species, tril, sigma, epsilon, cutoffs, e, s)
    return energy, -grad, dtril


def kinetic_energy(momenta, masses, system, n_systems):
    ke = np.zeros(n_systems)
    np.add.at(ke, np.asarray(system), 0.5 * np.sum(momenta**2, axis=-1) / masses)
    return ke


def maxwell_boltzmann(rng, masses, temperature):
    std = np.sqrt(masses * temperature * BOLTZMANN_CONSTANT)
    p = rng.standard_normal((masses.size, 3)) * std[:, None]
    return p - p.sum(axis=0) / masses.size


def _wrap_all(pos, system, tril):
    return wrap(pos, np.asarray(tril)[np.asarray(system)])


def velocity_verlet(pos, mom, forces, masses, system, species, tril, sigma, epsilon, cutoffs, dt, n_steps):
    """n_steps of VV; dt per system. Returns (pos, mom, forces, energies per step)."""
    dts = np.asarray(dt, dtype=np.float64)[np.asarray(system)][:, None]
    m = np.asarray(masses)[:, None]
    energies = []
    for _ in range(n_steps):
        mom = mom + forces * (dts / 2)
        pos = _wrap_all(pos + mom / m * dts, system, tril)
        e, forces, _ = lj_forces(pos, system, species, tril, sigma, epsilon, cutoffs)
        mom = mom + forces * (dts / 2)
        energies.append(e)
    return pos, mom, forces, np.array(energies)


def baoab(pos, mom, forces, masses, system, species, tril, sigma, epsilon, cutoffs, dt, temperature, friction, noise):
    """BAOAB steps with caller-provided standard-normal noise [n_steps, N, 3]."""
    sysi = np.asarray(system)
    dts = np.asarray(dt, dtype=np.float64)[sysi][:, None]
    m = np.asarray(masses)[:, None]
    c1 = np.exp(-np.asarray(friction)[sysi] * np.asarray(dt)[sysi])[:, None]
    c2 = np.sqrt(np.asarray(temperature)[sysi] * BOLTZMANN_CONSTANT * (1 - c1[:, 0] ** 2))[:, None]
    energies = []
    for eta in noise:
        mom = mom + forces * (dts / 2)
        pos = _wrap_all(pos + mom / m * (dts / 2), system, tril)
        mom = c1 * mom + c2 * np.sqrt(m) * eta
        pos = _wrap_all(pos + mom / m * (dts / 2), system, tril)
        e, forces, _ = lj_forces(pos, system, species, tril, sigma, epsilon, cutoffs)
        mom = mom + forces * (dts / 2)
        energies.append(e)
    return pos, mom, forces, np.array(energies)


def virial_stress(pos, grad, system, tril, dtril):
    """Cauchy stress per system, sigma_ab = -(sum_i r_ia dU/dr_ib + (h^T dU/dh)_ab) / V
    (observables/stress.py:70-82: ``position_gradients[:, None] * positions[..., None]``
    puts the position on the first index); h^T dU/dh uses the lower-triangular dU/dtril."""
    sysi = np.asarray(system)
    tril = np.asarray(tril, np.float64)
    out = np.zeros((tril.shape[0], 3, 3))
    np.add.at(out, sysi, np.asarray(pos)[:, :, None] * np.asarray(grad)[:, None, :])
    for s in range(tril.shape[0]):
        L = lattice_from_tril(tril[s])
        G = lattice_from_tril(np.asarray(dtril)[s])
        out[s] = -(out[s] + L.T @ G) / abs(np.linalg.det(L))
    return out


def instantaneous_pressure(ke, stress, tril):
    """P = 2K / 3V + Tr(sigma) / 3 per system (md/observables.py:38-61 with d = 3)."""
    tril = np.asarray(tril, np.float64)
    vol = np.abs(tril[:, 0] * tril[:, 2] * tril[:, 5])
    return 2.0 * np.asarray(ke) / (3.0 * vol) + np.trace(stress, axis1=1, axis2=2) / 3.0


def csvr_scale(mom, masses, system, n_systems, dt, temperature, tau, r1, r2):
    """CSVRStep (integrators.py:519-596) with caller-provided R1 ~ N(0, 1) and
    R2 ~ chi^2(N_dof - 1) per system; N_dof = 3 N - 3."""
    sysi = np.asarray(system)
    ke = kinetic_energy(mom, masses, sysi, n_systems)
    dof = 3.0 * np.bincount(sysi, minlength=n_systems) - 3.0
    kt = dof * np.asarray(temperature, np.float64) * BOLTZMANN_CONSTANT / 2
    c1 = np.exp(-np.asarray(dt, np.float64) / np.asarray(tau, np.float64))
    c2 = (1 - c1) * kt / (ke * dof)
    a2 = c1 + c2 * (np.asarray(r1) ** 2 + np.asarray(r2)) + 2 * np.asarray(r1) * np.sqrt(c1 * c2)
    return mom * np.sqrt(np.maximum(a2, 0.0))[sysi][:, None]


def cell_rescale_factor(pressure, tril, dt, temperature, target_pressure, tau_p, compressibility, min_scale, rp):
    """mu of StochasticCellRescalingStep (integrators.py:710-789) with caller-provided
    R ~ N(0, 1) per system."""
    tril = np.asarray(tril, np.float64)
    vol = np.abs(tril[:, 0] * tril[:, 2] * tril[:, 5])
    kt = np.asarray(temperature, np.float64) * BOLTZMANN_CONSTANT
    beta, tau_p, dt = (np.asarray(x, np.float64) for x in (compressibility, tau_p, dt))
    deps = dt / tau_p * beta * (pressure - np.asarray(target_pressure)) + np.sqrt(
        2.0 * kt * beta * dt / (tau_p * vol)) * np.asarray(rp)
    with np.errstate(over="ignore"):  # an overflowing exp is clipped like any other large mu
        return np.clip(np.exp(deps / 3.0), min_scale, 1.0 / np.asarray(min_scale, np.float64))


def csvr_npt(pos, mom, forces, masses, system, species, tril, sigma, epsilon, cutoffs, dt, temperature, tau,
             target_pressure, tau_p, compressibility, min_scale, r1, r2, rp, barostat=True):
    """make_csvr_npt_step (integrators.py:801-890; barostat=False: make_csvr_step, :598-640)
    with noise per step and system r1, r2, rp [n_steps, S].  Returns (pos, mom, forces, tril,
    energies [n_steps, S], pressures [n_steps, S]) — the pressure the barostat saw."""
    sysi = np.asarray(system)
    tril = np.array(tril, np.float64)
    ns = tril.shape[0]
    dts = np.asarray(dt, dtype=np.float64)[sysi][:, None]
    m = np.asarray(masses)[:, None]
    energies, pressures = [], []
    for t in range(len(r1)):
        mom = csvr_scale(mom, masses, sysi, ns, dt, temperature, tau, r1[t], r2[t])
        mom = mom + forces * (dts / 2)
        pos = _wrap_all(pos + mom / m * dts, sysi, tril)
        e, forces, dtr = lj_forces(pos, sysi, species, tril, sigma, epsilon, cutoffs)
        mom = mom + forces * (dts / 2)
        if barostat:
            ke = kinetic_energy(mom, masses, sysi, ns)
            prs = instantaneous_pressure(ke, virial_stress(pos, -forces, sysi, tril, dtr), tril)
            mu = cell_rescale_factor(prs, tril, dt, temperature, target_pressure, tau_p, compressibility,
                                     min_scale, rp[t])
            tril = tril * mu[:, None]
            pos = pos * mu[sysi][:, None]
            e, forces, _ = lj_forces(pos, sysi, species, tril, sigma, epsilon, cutoffs)
            pressures.append(prs)
        energies.append(e)
    return pos, mom, forces, tril, np.array(energies), np.array(pressures)
