"""Molecular-dynamics integrators in float64 (oracle, test infrastructure).

Restates src/kups/md/integrators.py: ``MomentumStep`` (:217-263, B:
p += F dt), ``PositionStep`` with ``MinimumImageConventionFlow`` (:104-211, A:
r += p/m dt then wrap into fractional [-0.5, 0.5)), ``StochasticStep``
(:330-401, O: p = e^{-gamma dt} p + sqrt(kT (1 - e^{-2 gamma dt})) sqrt(m) eta),
``make_velocity_verlet_step`` (:273-318: B(dt/2) A(dt) F B(dt/2)) and
``make_baoab_langevin_step`` (:405-455: B(dt/2) A(dt/2) O(dt) A(dt/2) F B(dt/2));
kinetic energy (src/kups/md/observables.py:17-35) and the Maxwell-Boltzmann
initialisation with centre-of-mass drift removal (application/md/data.py:170-176).
Forces are -dE/dx from the Lennard-Jones oracle over the reference-exact
neighbour list, rebuilt every step as the reference's MD app does.
"""

from __future__ import annotations

import numpy as np

from .lennard_jones import lj_from_edges
from .neighborlist import neighbor_list
from .unitcell import wrap
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
