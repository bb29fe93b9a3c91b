"""Seeded synthetic inputs with the shapes of the benchmark configurations.

* ``argon_fcc``: LJ argon on an FCC lattice (864 atoms = 6x6x6 cells, a = 5.74 A).
* ``batched_uneven_lj``: many independent cubic LJ systems with atom counts
  drawn uniformly from [n_min, n_max], reduced densities from U[rho_min,
  rho_max] sigma^-3 and temperatures from U[t_min, t_max] K.  Positions are a
  random subset of the sites of a simple-cubic lattice of spacing a >= the
  minimum separation d, each displaced by at most (a - d)/2 per axis, which
  guarantees every pair is at least d apart while staying seeded and fast.
* ``ionic_melt``: +1/-1 point ions with per-species LJ in a cubic box, same
  non-overlap construction.

Maxwell-Boltzmann momenta with the centre-of-mass drift removed follow
src/kups/application/md/data.py:170-176.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .units import BOLTZMANN_CONSTANT, FEMTO_SECOND

ARGON_SIGMA = 3.405
ARGON_EPS = 119.8 * BOLTZMANN_CONSTANT
ARGON_MASS = 39.948


@dataclass
class MDWorkload:
    positions: np.ndarray  # f64 [N, 3]
    momenta: np.ndarray  # f64 [N, 3]
    masses: np.ndarray  # f64 [N]
    species: np.ndarray  # int32 [N]
    system: np.ndarray  # int32 [N]
    tril: np.ndarray  # f64 [S, 6]
    temperature: np.ndarray  # K [S]
    time_step: np.ndarray  # internal units [S]
    friction: np.ndarray  # 1/internal time [S]
    sigma: np.ndarray  # [T, T]
    epsilon: np.ndarray  # [T, T]
    cutoff: float
    skin: float
    charges: np.ndarray | None = None

    @property
    def n_atoms(self) -> int:
        return int(self.positions.shape[0])

    @property
    def n_systems(self) -> int:
        return int(self.tril.shape[0])

    def select(self, systems) -> "MDWorkload":
        """The given systems (any order, no repeats), renumbered 0.. in that order, atoms grouped by system."""
        systems = np.asarray(systems, np.int64)
        parts = [np.nonzero(self.system == s)[0] for s in systems]
        idx = np.concatenate(parts)
        new_sys = np.repeat(np.arange(len(systems), dtype=np.int32), [len(p) for p in parts])
        return MDWorkload(self.positions[idx], self.momenta[idx], self.masses[idx], self.species[idx], new_sys,
                          self.tril[systems], self.temperature[systems], self.time_step[systems],
                          self.friction[systems], self.sigma, self.epsilon, self.cutoff, self.skin,
                          None if self.charges is None else self.charges[idx])

    def subset(self, lo: int, hi: int) -> "MDWorkload":
        """Systems [lo, hi) (atoms grouped by system), renumbered from 0."""
        sel = (self.system >= lo) & (self.system < hi)
        return MDWorkload(self.positions[sel], self.momenta[sel], self.masses[sel], self.species[sel],
                          (self.system[sel] - lo).astype(np.int32), self.tril[lo:hi], self.temperature[lo:hi],
                          self.time_step[lo:hi], self.friction[lo:hi], self.sigma, self.epsilon, self.cutoff, self.skin,
                          None if self.charges is None else self.charges[sel])


def _mb_momenta(rng, masses, kT, system, n_sys):
    std = np.sqrt(masses * kT[system])
    p = rng.standard_normal((masses.size, 3)) * std[:, None]
    cnt = np.bincount(system, minlength=n_sys).astype(np.float64)
    drift = np.stack([np.bincount(system, weights=p[:, a], minlength=n_sys) for a in range(3)], -1)
    return p - (drift / np.maximum(cnt, 1)[:, None])[system]


_BASES = {
    "sc": (np.zeros((1, 3)), 1.0),
    "bcc": (np.array([[0, 0, 0], [0.5, 0.5, 0.5]]), math.sqrt(3) / 2),
    "fcc": (np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]), 1 / math.sqrt(2)),
}


def lattice_positions(rng, n, box, dmin):
    """n points in a cubic box (centred at 0), pairwise >= dmin apart under PBC.

    Sites of whichever of the sc / bcc / fcc lattices (with the fewest cells
    holding n sites) has the largest nearest-neighbour spacing; a random subset
    of n sites, each jittered by at most (spacing - dmin) / 2 per axis.
    """
    best = None
    for base, nn_factor in _BASES.values():
        k = max(1, int(math.ceil((n / len(base)) ** (1 / 3))))
        while len(base) * k**3 < n:
            k += 1
        nn = box / k * nn_factor
        if best is None or nn > best[0]:
            best = (nn, k, base)
    nn, k, base = best
    if nn < dmin:
        raise ValueError("box too small for the minimum separation")
    cells = np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), -1).reshape(-1, 1, 3)
    sites = (cells + base[None]).reshape(-1, 3) / k * box
    pick = rng.choice(sites.shape[0], size=n, replace=False)
    jitter = (nn - dmin) / 2.0 / math.sqrt(3)
    return sites[pick] + rng.uniform(-jitter, jitter, (n, 3)) - box / 2


def argon_fcc(n_side=6, a=5.74, temperature=94.4, dt_fs=2.0, friction_per_ps=1.0, cutoff=8.5, skin=1.0, seed=0):
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.array([(i, j, k) for i in range(n_side) for j in range(n_side) for k in range(n_side)])
    frac = ((g[:, None, :] + base[None]) / n_side).reshape(-1, 3) - 0.5
    L = n_side * a
    pos = frac * L
    n = pos.shape[0]
    masses = np.full(n, ARGON_MASS)
    system = np.zeros(n, np.int32)
    T = np.array([temperature])
    mom = _mb_momenta(rng, masses, T * BOLTZMANN_CONSTANT, system, 1)
    return MDWorkload(pos, mom, masses, np.zeros(n, np.int32), system, np.array([[L, 0, L, 0, 0, L]], float), T,
                      np.array([dt_fs * FEMTO_SECOND]), np.array([friction_per_ps / 1000.0 / FEMTO_SECOND]),
                      np.array([[ARGON_SIGMA]]), np.array([[ARGON_EPS]]), cutoff, skin)


def batched_uneven_lj(n_systems=4096, n_min=64, n_max=2048, rho_min=0.7, rho_max=0.9, t_min=80.0, t_max=140.0,
                      rc_sigma=2.5, skin_sigma=0.3, dt_fs=2.0, friction_per_ps=1.0, min_sep_sigma=0.9, seed=1):
    rng = np.random.default_rng(seed)
    counts = rng.integers(n_min, n_max + 1, n_systems)
    rho = rng.uniform(rho_min, rho_max, n_systems)
    temps = rng.uniform(t_min, t_max, n_systems)
    boxes = (counts / rho) ** (1 / 3) * ARGON_SIGMA
    pos = np.concatenate([lattice_positions(rng, int(c), float(b), min_sep_sigma * ARGON_SIGMA)
                          for c, b in zip(counts, boxes)])
    system = np.repeat(np.arange(n_systems, dtype=np.int32), counts)
    masses = np.full(pos.shape[0], ARGON_MASS)
    mom = _mb_momenta(rng, masses, temps * BOLTZMANN_CONSTANT, system, n_systems)
    tril = np.zeros((n_systems, 6))
    tril[:, 0] = tril[:, 2] = tril[:, 5] = boxes
    return MDWorkload(pos, mom, masses, np.zeros(pos.shape[0], np.int32), system, tril, temps,
                      np.full(n_systems, dt_fs * FEMTO_SECOND), np.full(n_systems, friction_per_ps / 1000.0 / FEMTO_SECOND),
                      np.array([[ARGON_SIGMA]]), np.array([[ARGON_EPS]]), rc_sigma * ARGON_SIGMA, skin_sigma * ARGON_SIGMA)


@dataclass
class IonicMelt:
    positions: np.ndarray  # f64 [N, 3]
    momenta: np.ndarray
    masses: np.ndarray
    charges: np.ndarray
    species: np.ndarray  # 0 = cation, 1 = anion
    tril: np.ndarray  # [1, 6]
    sigma: np.ndarray  # [2, 2] Lorentz-Berthelot
    epsilon: np.ndarray
    cutoff: float
    alpha: float
    kvec_n: np.ndarray  # [1, n_k, 3]
    time_step: float


def ionic_melt(n_ions=4000, box=40.0, min_sep=2.2, temperature=1200.0, dt_fs=1.0, cutoff=12.0, alpha=0.3, kmax=8,
               seed=2):
    """+1/-1 point ions with per-species LJ (eps 0.1 / 0.15 kcal/mol, sigma 2.35 / 4.40 A, LB mixing) in
    a cubic box; k vectors = the half-space integer box |n|_inf <= kmax (n_x >= 0).  Masses (not given by
    the configuration) are those of Na and Cl, 22.99 and 35.45 u."""
    from .units import KILO_CALORIE, MOL

    rng = np.random.default_rng(seed)
    pos = lattice_positions(rng, n_ions, box, min_sep)
    species = (np.arange(n_ions) % 2).astype(np.int32)
    charges = np.where(species == 0, 1.0, -1.0)
    masses = np.where(species == 0, 22.99, 35.45)
    kcal = KILO_CALORIE / MOL
    s = np.array([2.35, 4.40])
    e = np.array([0.1, 0.15]) * kcal
    sigma, epsilon = (s[:, None] + s) / 2, np.sqrt(e[:, None] * e)
    system = np.zeros(n_ions, np.int32)
    mom = _mb_momenta(rng, masses, np.array([temperature * BOLTZMANN_CONSTANT]), system, 1)
    m = int(kmax)
    kn = np.stack(np.meshgrid(np.arange(0, m + 1), np.arange(-m, m + 1), np.arange(-m, m + 1)), -1).reshape(-1, 3)
    return IonicMelt(pos, mom, masses, charges, species, np.array([[box, 0, box, 0, 0, box]], float), sigma, epsilon,
                     cutoff, alpha, kn[None].astype(np.int32), dt_fs * FEMTO_SECOND)


def porous_framework(rng, tril, n_atoms, channel_radius=6.0, jitter=0.2):
    """Rigid host: a random subset of a fractional grid outside a cylindrical channel
    along c through the origin, positions wrapped into the primary cell [-0.5, 0.5) as
    the reference's host loader leaves them when it builds a supercell
    (src/kups/application/mcmc/data.py:368-371).  The wrap matters: when some axes need
    several periodic images and others one, the reference's pair search applies the
    image offsets to the raw fractional difference (core/neighborlist.py:542-564,
    595-624), so along a one-image axis only atoms stored in the same period as a guest
    (guests are wrapped into [-0.5, 0.5) by every move) are seen.
    2000 sites at >= 2.8 A separation do not fit in a 25 A, 120 degree cell (packing
    fraction above one), so the grid spacing is the densest that leaves the channel
    empty."""
    t = np.asarray(tril, float)
    L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
    n = 8
    while True:
        g = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
        f = (g + 0.5) / n
        d = f[:, :2] - 0.5
        d -= np.round(d)
        cart = np.concatenate([d, np.zeros((len(d), 1))], 1) @ L
        keep = np.hypot(cart[:, 0], cart[:, 1]) > channel_radius
        if keep.sum() >= n_atoms:
            break
        n += 1
    f = f[keep] - 0.5  # channel axis at the origin
    pick = rng.choice(len(f), size=n_atoms, replace=False)
    f = f[pick] + rng.uniform(-1, 1, (n_atoms, 3)) * (jitter / np.array([t[0], t[2], t[5]]))
    return ((f + 0.5) % 1.0 - 0.5) @ L


def replicate_host(positions, tril, reps):
    """Supercell of a host, as the reference's HostConfig.unitcell_replication builds it
    (core/unitcell.py:196-244, 477-506): cell rows scaled by the multiplicities, copies
    shifted by integer lattice vectors and wrapped into the new primary cell [-0.5, 0.5)."""
    t = np.asarray(tril, float)
    L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
    shifts = np.stack(np.meshgrid(*[np.arange(m) for m in reps], indexing="ij"), -1).reshape(-1, 3)
    m = np.asarray(reps, float)
    t2 = t * np.array([m[0], m[1], m[1], m[2], m[2], m[2]])
    L2 = L * m[:, None]
    pos = (np.asarray(positions, float)[None] + (shifts @ L)[:, None]).reshape(-1, 3)
    f = pos @ np.linalg.inv(L2)
    return ((f + 0.5) % 1.0 - 0.5) @ L2, t2


def gcmc_co2_framework(n_replicas=1024, n_fw=2000, p_min_bar=0.1, p_max_bar=10.0, temperature=298.0, rc=12.0,
                       alpha=0.25, precision=1e-6, max_mol=192, seed=3, replicate=(2, 2, 1), eps_scale=1.0,
                       charge_scale=1.0):
    """Rigid 3-site CO2 in a synthetic rigid framework (4 LJ types, Gaussian charges shifted
    to net zero), replicas at log-spaced pressures; critical constants of CO2 for the
    Peng-Robinson fugacity: Tc 303.75 K, Pc 7.84 MPa, omega 0.22394.

    The host's cell (25 A, 90/90/120 degrees) has perpendicular widths 21.65, 21.65 and
    25 A, so with a 12 A cutoff the reference's pair search needs three images along a
    and b and one along c, and in that mixed case it applies the image offsets to raw
    fractional differences: every pair across the c faces is missed and guests overlap
    there without bound.  ``replicate`` (the reference's unitcell_replication) builds
    the simulation box from copies of the host cell; (2, 2, 1) makes every width at
    least twice the cutoff, so every pair is found by minimum image.  ``replicate=None``
    keeps the single cell (the reference's mixed-image behaviour, used by the parity
    tests).  ``eps_scale`` / ``charge_scale`` weaken the host (test systems that
    equilibrate quickly)."""
    from . import gcmc
    from .ewald import kvecs_from_kmax
    from .units import PASCAL

    rng = np.random.default_rng(seed)
    L = np.array([[25.0, 0, 0], [25.0 * np.cos(np.radians(120)), 25.0 * np.sin(np.radians(120)), 0],
                  [0, 0, 25.0]])
    tril = np.array([L[0, 0], L[1, 0], L[1, 1], L[2, 0], L[2, 1], L[2, 2]])
    fw = porous_framework(rng, tril, n_fw)
    fw_sp = rng.integers(0, 4, n_fw)
    q = rng.normal(0, 0.3, n_fw)
    q = (q - q.mean()) * charge_scale
    if replicate is not None and tuple(replicate) != (1, 1, 1):
        k = int(np.prod(replicate))
        fw, tril = replicate_host(fw, tril, replicate)
        fw_sp, q = np.tile(fw_sp, k), np.tile(q, k)
        n_fw = len(fw)
    sig = np.concatenate([rng.uniform(2.5, 3.5, 4), [2.80, 3.05]])
    eps = np.concatenate([rng.uniform(20, 80, 4) * eps_scale, [27.0, 79.0]]) * BOLTZMANN_CONSTANT
    sigma, epsilon = gcmc.lorentz_berthelot(sig, eps)
    kmax = 2 * alpha * np.sqrt(-np.log(precision / 2))
    kn = kvecs_from_kmax(tril, kmax)
    pressures = np.logspace(np.log10(p_min_bar), np.log10(p_max_bar), n_replicas) * 1e5
    kT = temperature * BOLTZMANN_CONSTANT
    # ln(f / kT) with f from the Peng-Robinson fugacity in Pa, converted to eV / A^3
    la = np.array([gcmc.peng_robinson_log_fugacity(p, temperature, 7.84e6, 303.75, 0.22394).log_fugacity[0]
                   + np.log(PASCAL) - np.log(kT) for p in pressures])
    S = n_replicas
    return gcmc.GCMCSetup(
        fw_positions=fw, fw_species=fw_sp, fw_charges=q, fw_start=np.zeros(S, int), fw_count=np.full(S, n_fw),
        tril=np.repeat(tril[None], S, 0),
        motif_positions=np.array([[0.0, 0, 0], [1.16, 0, 0], [-1.16, 0, 0]]), motif_species=np.array([4, 5, 5]),
        motif_charges=np.array([0.70, -0.35, -0.35]), sigma=sigma, epsilon=epsilon, rc_lj=np.full(S, rc),
        rc_ew=np.full(S, rc), alpha=np.full(S, alpha), kvec_n=np.repeat(kn[None], S, 0),
        temperature=np.full(S, temperature), log_activity=la, max_mol=max_mol, tail_correction=True)
