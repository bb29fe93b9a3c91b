"""Monte Carlo move generator, muVT acceptance and step-width scheduler in float64 (oracle,
test infrastructure).

Restates, for checking the GPU GCMC step of ``kups_gcmc_run``:

* the muVT log acceptance ratio: ``BoltzmannLogProbabilityRatio`` (src/kups/mcmc/probability.py:60-109,
  ln p = (U_old - U_new) / kT), ``LogFugacityRatio`` (:116-173, sum over species of
  (N' - N) ln(a V) + ln(N! / N'!), zero where N' == N) and ``MuVTLogProbabilityRatio`` (:176-225,
  their sum); ``log_factorial_ratio`` (src/kups/core/utils/math.py:21-41, lgamma(N + 1) - lgamma(M + 1));
* the unit quaternion of ``Quaternion.random`` (Shoemake; src/kups/core/utils/quaternion.py:71-98),
  its power (:182-208, ``_pow_quaternion``), product and rotation matrix (``_multiply_quaternions``,
  ``_quat_to_mat``) and ``point @ q`` = R point (:119-151);
* the rigid-molecule moves of ``make_gcmc_mcmc_propagator`` (src/kups/mcmc/moves.py:1078-1230):
  translation by N(0, 1) width per axis then wrap (:222-244, :200-219), rotation by q ** width about
  the atom mean unwrapped against one atom (:158-197, :247-265; ``center_of_mass`` of
  src/kups/core/utils/position.py:22-85 without weights), reinsertion (full rotation, uniform
  fractional offset, wrap; :268-295), insertion of the template rotated and shifted by a uniform
  fractional offset (:573-675) and deletion of a chosen molecule (:678-773);
* ``acceptance_target_schedule`` (src/kups/core/parameter_scheduler.py:161-208) with the defaults of
  ``ParameterSchedulerState.create`` (:103-160: target 0.5, tolerance 0.05, multiplicity 1.1,
  negative correlation, 100-move history, bounds [0, upper]).

The GPU draws its randomness from Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random
numbers: as easy as 1, 2, 3", SC'11) keyed by the seed, with stream and counter as the kernel
assigns them; ``philox4x32_10`` restates that published generator so the replay can regenerate
every proposal and uniform of a GPU run (the reference's JAX keys are not reproduced: its keys
and the GPU's Philox streams are different generators of the same distributions).
"""

from __future__ import annotations

import math

import numpy as np

from .units import BOLTZMANN_CONSTANT
from .unitcell import lattice_from_tril, to_fractional

_M0, _M1 = 0xD2511F53, 0xCD9E8D57
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


# ----------------------------------------------------------------------------- generator
def philox4x32_10(ctr, k0, k1):
    """Philox4x32 with ten rounds: ctr = (x, y, z, w) 32-bit words, key (k0, k1)."""
    x, y, z, w = (int(c) & _MASK for c in ctr)
    k0, k1 = int(k0) & _MASK, int(k1) & _MASK
    for _ in range(10):
        p0, p1 = _M0 * x, _M1 * z
        x, y, z, w = ((p1 >> 32) ^ y ^ k0) & _MASK, p1 & _MASK, ((p0 >> 32) ^ w ^ k1) & _MASK, p0 & _MASK
        k0, k1 = (k0 + _W0) & _MASK, (k1 + _W1) & _MASK
    return x, y, z, w


def rng4(seed, stream, counter):
    """The four words of one Philox block: counter in words 0-1, stream in words 2-3, key = seed."""
    seed, stream, counter = int(seed), int(stream), int(counter)
    return philox4x32_10((counter & _MASK, counter >> 32, stream & _MASK, stream >> 32), seed & _MASK,
                         (seed >> 32) & _MASK)


def u01(v):
    """Uniform in [0, 1) from the top 24 bits of a word."""
    return (int(v) >> 8) * (1.0 / 16777216.0)


def u01_open0(v):
    """Uniform in (0, 1] from the top 24 bits of a word."""
    return (int(v) >> 8) * (1.0 / 16777216.0) + 1.0 / 16777216.0


def normal4(seed, stream, counter):
    """Four standard normals by the Box-Muller transform of one Philox block."""
    x, y, z, w = rng4(seed, stream, counter)
    m1 = math.sqrt(-2.0 * math.log(u01_open0(x)))
    m2 = math.sqrt(-2.0 * math.log(u01_open0(z)))
    a1, a2 = 2.0 * math.pi * u01_open0(y), 2.0 * math.pi * u01_open0(w)
    return np.array([m1 * math.cos(a1), m1 * math.sin(a1), m2 * math.cos(a2), m2 * math.sin(a2)])


# ----------------------------------------------------------------------------- quaternions
def shoemake(u1, u2, u3):
    """(w, x, y, z) of a uniformly distributed rotation from three uniforms (quaternion.py:71-98)."""
    a, b = math.sqrt(1.0 - u1), math.sqrt(u1)
    return np.array([a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2),
                     b * math.sin(2 * math.pi * u3), b * math.cos(2 * math.pi * u3)])


def qmul(q1, q2):
    """Hamilton product (``_multiply_quaternions``)."""
    w1, x1, y1, z1 = q1
    w2, x2, y2, z2 = q2
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def qpow(q, e):
    """q ** e: the same axis, the angle times e; the identity stays the identity (``_pow_quaternion``)."""
    q = np.asarray(q, np.float64)
    if q[0] < 0:
        q = -q
    angle = 2.0 * math.acos(min(max(q[0], -1.0), 1.0))
    s = float(np.linalg.norm(q[1:]))
    axis = q[1:] / (s if s > 1e-10 else 1.0)
    half = 0.5 * angle * e
    return np.concatenate([[math.cos(half)], axis * math.sin(half)])


def quat_matrix(q):
    """Rotation matrix of a unit quaternion (``_quat_to_mat``)."""
    w, x, y, z = q
    return np.array([[x * x - y * y - z * z + w * w, 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), -x * x + y * y - z * z + w * w, 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), -x * x - y * y + z * z + w * w]])


def rotate(points, q):
    """``points @ q``: each point multiplied by the rotation matrix, R p (quaternion.py:119-151)."""
    return np.asarray(points, np.float64) @ quat_matrix(q).T


# ----------------------------------------------------------------------------- acceptance
def log_factorial_ratio(n, m):
    """ln(N! / M!) = lgamma(N + 1) - lgamma(M + 1), elementwise."""
    n, m = np.asarray(n, np.float64), np.asarray(m, np.float64)
    lg = np.vectorize(math.lgamma)
    return lg(n + 1.0) - lg(m + 1.0)


def boltzmann_log_ratio(old_energy, new_energy, temperature):
    """(U_old - U_new) / (k_B T) per system."""
    return (np.asarray(old_energy, np.float64) - np.asarray(new_energy, np.float64)) / (
        np.asarray(temperature, np.float64) * BOLTZMANN_CONSTANT)


def log_fugacity_ratio(log_activity, volume, counts, patched_counts):
    """sum over species of (N' - N) (ln a + ln V) + ln(N! / N'!), 0 for species whose count is
    unchanged; arrays [S, species] (volume [S])."""
    la = np.atleast_2d(np.asarray(log_activity, np.float64))
    c = np.atleast_2d(np.asarray(counts, np.float64))
    pc = np.atleast_2d(np.asarray(patched_counts, np.float64))
    ln_fv = la + np.log(np.asarray(volume, np.float64))[:, None]
    r = (pc - c) * ln_fv + log_factorial_ratio(c, pc)
    return np.where(pc == c, 0.0, r).sum(-1)


def muvt_log_ratio(old_energy, new_energy, temperature, log_activity, volume, counts, patched_counts):
    """ln acc of the muVT ensemble: the Boltzmann term plus the fugacity term."""
    return boltzmann_log_ratio(old_energy, new_energy, temperature) + log_fugacity_ratio(
        log_activity, volume, counts, patched_counts)


# ----------------------------------------------------------------------------- step widths
class AcceptanceScheduler:
    """``acceptance_target_schedule`` for one system and one move: record the decision in a
    circular history; when the history index returns to zero, compare the history mean with
    the target and, outside the dead band |mean - target| <= tolerance, scale the value by the
    multiplicity m: with negative correlation (step widths) by 1 / m when the mean is below the
    target and by m otherwise, with positive correlation the other way round; then clip to
    [lower, upper] (None: unbounded)."""

    def __init__(self, value=0.1, multiplicity=1.1, target=0.5, tolerance=0.05, lower=0.0, upper=None,
                 history_length=100, positive=False):
        self.value = float(value)
        self.mult, self.target, self.tol = float(multiplicity), float(target), float(tolerance)
        self.lower, self.upper, self.positive = lower, upper, bool(positive)
        self.history = np.zeros(history_length)
        self.index = 0

    def __call__(self, accepted) -> float:
        self.history[self.index] = float(accepted)
        self.index = (self.index + 1) % len(self.history)
        avg = float(self.history.mean())
        m = self.mult if self.positive else 1.0 / self.mult
        new = self.value * m if avg < self.target else self.value / m
        if self.lower is not None:
            new = max(new, float(self.lower))
        if self.upper is not None:
            new = min(new, float(self.upper))
        if abs(avg - self.target) > self.tol and self.index == 0:
            self.value = new
        return self.value


# ----------------------------------------------------------------------------- geometry helpers
def _wrap(x, L, Linv):
    f = np.asarray(x, np.float64) @ Linv
    f = (f + 0.5) - np.floor(f + 0.5) - 0.5
    return f @ L


def atom_mean(pos, L, Linv):
    """Mean of a molecule's atoms unwrapped against its first atom, wrapped into the cell."""
    p = np.asarray(pos, np.float64)
    d = _wrap(p - p[0], L, Linv)
    return _wrap(p[0] + d.mean(0), L, Linv)


# ----------------------------------------------------------------------------- the GPU step's proposals
MOVES = ("translate", "rotate", "reinsert", "insert", "delete")


def move_kind(seed, counter, move_cum):
    """The move of a step, shared by every system: the first of translate / rotate / reinsert whose
    cumulative probability exceeds u, else exchange, whose insert / delete coin is the low bit of
    the second word (one draw per step for the whole batch, as propose_mixed and the exchange coin
    of moves.py:1217 make one choice per call)."""
    x, y, _, _ = rng4(seed, 0, counter)
    u = u01(x)
    k = 0
    while k < 3 and u >= float(np.float32(move_cum[k])):
        k += 1
    if k == 3:
        k = 4 if (y & 1) else 3
    return k


def propose(seed, counter, system, kind, n_mol, mol_positions, motif, width, tril):
    """Float64 restatement of the proposal the GPU makes for one system in one step.

    ``mol_positions`` [n_mol, apm, 3] are the current molecules (Cartesian), ``motif`` [apm, 3]
    the insertion template, ``width`` the scheduler value of the move.  Returns
    (mol, new [apm, 3] or None, has_old): translation and rotation move molecule
    r1.x mod n_mol, reinsertion re-places it with a full rotation and a uniform fractional
    offset, insertion takes the next free slot, deletion removes molecule r1.x mod n_mol."""
    L = lattice_from_tril(np.asarray(tril, np.float64))
    Linv = np.linalg.inv(L)
    stream = 1 + int(system)
    r1 = rng4(seed, stream, 8 * counter)
    r2 = rng4(seed, stream, 8 * counter + 1)
    r3 = rng4(seed, stream, 8 * counter + 2)
    if kind == 3:
        q = shoemake(u01(r2[0]), u01(r2[1]), u01(r2[2]))
        shift = np.array([u01(r3[0]), u01(r3[1]), u01(r3[2])]) @ L
        return n_mol, _wrap(rotate(motif, q) + shift, L, Linv), False
    if n_mol == 0:
        return -1, None, False
    mol = r1[0] % n_mol
    old = np.asarray(mol_positions[mol], np.float64)
    if kind == 4:
        return mol, None, True
    if kind == 0:
        eta = normal4(seed, stream, 8 * counter + 3)[:3]
        return mol, _wrap(old + eta * width, L, Linv), True
    q = shoemake(u01(r2[0]), u01(r2[1]), u01(r2[2]))
    if kind == 1:
        q = qpow(q, width)
    com = atom_mean(old, L, Linv)
    rel = _wrap(old - com, L, Linv)
    new = _wrap(rotate(rel, q) + com, L, Linv)
    if kind == 2:
        new = _wrap(new + np.array([u01(r3[0]), u01(r3[1]), u01(r3[2])]) @ L, L, Linv)
    return mol, new, True


def log_uniform(seed, counter, system):
    """ln u of the step's acceptance uniform u in (0, 1] (24-bit grid)."""
    w = rng4(seed, 1 + int(system), 8 * counter + 4)[3]
    return math.log(((w >> 8) + 1.0) * (1.0 / 16777216.0))


def gcmc_log_acceptance(de, temperature, log_activity, volume, n_old, n_new, ln_proposal=0.0):
    """ln acc of one rigid-molecule move with one molecule species: -dE / kT + the fugacity term
    + the proposal's log ratio."""
    return float(-de / (temperature * BOLTZMANN_CONSTANT)
                 + log_fugacity_ratio([[log_activity]], [volume], [[n_old]], [[n_new]])[0] + ln_proposal)


def fractional(x, tril):
    return to_fractional(np.asarray(x, np.float64), np.asarray(tril, np.float64))
