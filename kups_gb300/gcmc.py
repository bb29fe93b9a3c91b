"""Batched GCMC of rigid molecules in rigid frameworks behind kUPS's MCMC propagator.

Mirrors the pieces of src/kups/application/simulations/mcmc_rigid.py the
GCMC run wires together (``init_state`` :310-382, ``make_propagator``
:281-307): the LJ + Ewald (with intramolecular exclusion) + LJ tail
potential, the muVT acceptance with the Peng-Robinson fugacity
(src/kups/mcmc/fugacity.py:38-193, application/mcmc/data.py:380-392) and
``make_gcmc_mcmc_propagator`` (src/kups/mcmc/moves.py:1078-1230) with one
adaptive step-width scheduler per move (``ParameterSchedulerState.create``,
src/kups/core/parameter_scheduler.py:103-160; translation bounded by half
the smallest cell width, mcmc_rigid.py:357-372).  Every MC step of every
system runs on the GPU (``kups_gcmc_run``); host code only sets up.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import NamedTuple

import numpy as np
import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status
from .units import BOLTZMANN_CONSTANT, PASCAL, TO_STANDARD_UNITS

MOVES = ("translate", "rotate", "reinsert", "insert", "delete")


# ----------------------------------------------------------------------------- host-side thermodynamics
class LogFugacityResult(NamedTuple):
    """ln f per component (in the pressure's unit) and the compressibility Z of the root each
    component's fugacity was taken from (``LogFugacityResult``, src/kups/mcmc/fugacity.py:23-32)."""

    log_fugacity: np.ndarray
    compressibility: np.ndarray


def peng_robinson_log_fugacity(pressure, temperature, critical_pressure, critical_temperature, acentric_factor,
                               composition=None, interaction=None) -> LogFugacityResult:
    """Peng-Robinson fugacity of each component of a gas mixture (src/kups/mcmc/fugacity.py:35-193).

    Reduced pressure and temperature per component, m(omega), A_i = 0.45724 Pr_i / Tr_i^2
    (1 + m_i (1 - sqrt(Tr_i)))^2, B_i = 0.0778 Pr_i / Tr_i; mixing A = sum_ij y_i y_j (1 - k_ij)
    sqrt(A_i A_j), B = sum_i y_i B_i; Z from the cubic Z^3 + (B - 1) Z^2 + (A - 3B^2 - 2B) Z -
    (AB - B^2 - B^3) = 0; for each component the real root with the smallest ln phi_i (the gas
    phase, as RASPA selects it) among roots where ln phi_i is defined (Z > B).  The pressure's
    unit cancels in every reduced quantity, so ln f is in that unit.  Host code (once per setup).
    """
    pc = np.atleast_1d(np.asarray(critical_pressure, np.float64))
    n = pc.size
    tc = np.atleast_1d(np.asarray(critical_temperature, np.float64))
    om = np.atleast_1d(np.asarray(acentric_factor, np.float64))
    y = np.ones(1) if composition is None else np.atleast_1d(np.asarray(composition, np.float64))
    kij = np.zeros((n, n)) if interaction is None else np.asarray(interaction, np.float64).reshape(n, n)
    if y.size != n:
        raise ValueError("composition needs one mole fraction per component")
    p, t = float(pressure), float(temperature)
    pr, tr = p / pc, t / tc
    m = 0.37464 + 1.54226 * om - 0.26992 * om**2
    sa = 1.0 + m * (1.0 - np.sqrt(tr))
    a = 0.45724 * pr / tr**2 * sa**2
    b = 0.0778 * pr / tr
    aij = (1.0 - kij) * np.sqrt(np.outer(a, a))
    bm = float(y @ b)
    am = float(y @ aij @ y)
    roots = np.roots([1.0, bm - 1.0, am - 3.0 * bm**2 - 2.0 * bm, -(am * bm - bm**2 - bm**3)])
    scale = max(1.0, float(np.max(np.abs(roots))))
    z = np.sort(roots[np.abs(roots.imag) <= 1e-10 * scale].real)
    sq2 = math.sqrt(2.0)
    da = 2.0 * aij @ y
    best_phi = np.full(n, np.inf)
    best_z = np.full(n, np.nan)
    for zr in z:
        if not (zr > bm and zr > 0.0):
            continue
        lnphi = ((b / bm) * (zr - 1.0) - math.log(zr - bm)
                 - am / (2.0 * sq2 * bm) * (da / am - b / bm)
                 * math.log((zr + (1.0 + sq2) * bm) / (zr + (1.0 - sq2) * bm)))
        better = lnphi < best_phi
        best_phi = np.where(better, lnphi, best_phi)
        best_z = np.where(better, zr, best_z)
    with np.errstate(divide="ignore"):
        ln_f = best_phi + math.log(p) + np.log(y)
    return LogFugacityResult(ln_f, best_z)


def lorentz_berthelot(sigma, epsilon):
    s, e = np.asarray(sigma, float), np.asarray(epsilon, float)
    return (s[:, None] + s) / 2, np.sqrt(e[:, None] * e)


def prefactor(tril, kvec_n, alpha):
    """P(k) = (2 - [n_x = 0]) 2 pi / V exp(-k^2 / 4 a^2) / k^2, 0 for k = 0 (ewald.py:363-391)."""
    t = np.asarray(tril, float)
    L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
    inv = np.linalg.inv(L)
    k = 2 * np.pi * np.asarray(kvec_n, float) @ inv.T
    k2 = (k * k).sum(-1)
    vol = abs(t[0] * t[2] * t[5])
    with np.errstate(divide="ignore", invalid="ignore"):
        p = (2 - (np.asarray(kvec_n)[:, 0] == 0)) * 2 * np.pi / vol * np.exp(-k2 / (4 * alpha**2)) / k2
    return np.where(k2 > 0, p, 0.0)


# ----------------------------------------------------------------------------- state
@dataclass
class GCMCSetup:
    """Host description of a batch of GCMC systems sharing one molecule species."""

    fw_positions: np.ndarray  # [F, 3] Cartesian, as stored (no wrap applied)
    fw_species: np.ndarray  # [F]
    fw_charges: np.ndarray  # [F]
    fw_start: np.ndarray  # [S]
    fw_count: np.ndarray  # [S]
    tril: np.ndarray  # [S, 6]
    motif_positions: np.ndarray  # [apm, 3] template
    motif_species: np.ndarray  # [apm]
    motif_charges: np.ndarray  # [apm]
    sigma: np.ndarray  # [T, T]
    epsilon: np.ndarray  # [T, T]
    rc_lj: np.ndarray  # [S]
    rc_ew: np.ndarray  # [S]
    alpha: np.ndarray  # [S]
    kvec_n: np.ndarray  # [S, nk, 3]
    temperature: np.ndarray  # [S] K
    log_activity: np.ndarray  # [S] ln(f / kT), 1 / A^3
    max_mol: int = 64
    tail_correction: bool = True
    move_weights: tuple = (1.0, 1.0, 1.0, 2.0)  # translate, rotate, reinsert, exchange

    @property
    def n_systems(self) -> int:
        return int(self.tril.shape[0])


def exclusion_energy_of_molecule(pos, q, alpha):
    """sum over intramolecular pairs of K q_a q_b (erfc(alpha r) - 1) / r (ewald.py:328-346)."""
    from scipy.special import erfc

    e = 0.0
    for a in range(len(q)):
        for b in range(a + 1, len(q)):
            r = float(np.linalg.norm(pos[a] - pos[b]))
            e += TO_STANDARD_UNITS * q[a] * q[b] * (erfc(alpha * r) - 1.0) / r
    return e


def tail_coefficients(sigma, epsilon, rc, volume, enabled=True):
    """(8/3) pi eps sigma^3 [(sigma/rc)^9/3 - (sigma/rc)^3] / V per species pair (lennard_jones.py:276-315)."""
    t1 = (sigma / rc) ** 3
    c = (8 / 3) * np.pi * epsilon * sigma**3 * (t1**3 / 3 - t1) / volume
    return np.where(epsilon > 0, c, 0.0) if enabled else np.zeros_like(c)


def _morton_order(pos, tril, cell=3.2):
    """Permutation putting host atoms in Z-order of ~``cell`` A cells, so the 32 atoms a warp
    reads lie close together and agree on being inside or outside the cutoff."""
    t = np.asarray(tril, float)
    L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
    f = np.asarray(pos, float) @ np.linalg.inv(L)
    f -= np.floor(f)
    vol = abs(np.linalg.det(L))
    w = np.array([vol / np.linalg.norm(np.cross(L[(a + 1) % 3], L[(a + 2) % 3])) for a in range(3)])
    n = np.maximum(1, np.floor(w / cell)).astype(np.int64)
    c = np.minimum((f * n).astype(np.int64), n - 1)
    key = np.zeros(len(c), np.int64)
    for bit in range(10):
        for a in range(3):
            key |= ((c[:, a] >> bit) & 1) << (3 * bit + a)
    return np.argsort(key, kind="stable")


def _group_bounds(pos, tril, one_cell, n_groups):
    """[n_groups, 2, 4] per 32 consecutive atoms: fractional centre (circular mean, in
    [-0.5, 0.5)) and per-axis half extents (circular distance to the centre, + 1e-5).  A block
    used with several different cells gets half extents of 1 (its groups are never skipped)."""
    out = np.zeros((n_groups, 2, 4))
    out[:, 1, :3] = 1.0
    if not one_cell or len(pos) == 0:
        return out
    t = np.asarray(tril, float)
    L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
    f = np.asarray(pos, float) @ np.linalg.inv(L)
    for g in range(n_groups):
        fg = f[32 * g:32 * g + 32]
        if len(fg) == 0:
            continue
        d = fg - fg[0]
        d -= np.round(d)
        c = fg[0] + d.mean(0)
        c -= np.round(c)
        e = fg - c
        e -= np.round(e)
        out[g, 0, :3] = c
        out[g, 1, :3] = np.abs(e).max(0) + 1e-5
    return out


class GCMC:
    """Device state + the propagator ``__call__(key, n_steps)``."""

    def __init__(self, setup: GCMCSetup, seed: int = 0):
        self.setup = setup
        s = setup.n_systems
        apm = len(setup.motif_charges)
        T = setup.sigma.shape[0]
        if not (1 <= apm <= 8 and 1 <= T <= 8):
            raise ValueError("GCMC supports 1..8 atoms per molecule and 1..8 species")
        for name, sp in (("framework", setup.fw_species), ("motif", setup.motif_species)):
            if len(sp) and (np.min(sp) < 0 or np.max(sp) >= T):
                raise ValueError(f"{name} species outside the {T} parameter rows")
        if setup.kvec_n.shape[1] > 4096 or np.abs(setup.kvec_n).max() > 16:
            raise ValueError("at most 4096 k vectors with |n| <= 16 per axis")
        dev = "cuda"
        f32 = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device=dev)
        f64 = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)
        i32 = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.int32, device=dev)
        sp_bits = lambda sp: np.asarray(sp, np.int32).view(np.float32)
        # host atoms of each block in spatial (Z) order on the device, each block starting on a
        # multiple of 32 atoms, with a bounding table per 32 atoms (fw_group); energies do not
        # depend on the order, only the float32 summation order does
        pos_d, q_d, sp_d, grp, starts = [], [], [], [], {}
        off = 0
        for a0, n in sorted(set(zip(setup.fw_start.tolist(), setup.fw_count.tolist()))):
            users = np.nonzero((setup.fw_start == a0) & (setup.fw_count == n))[0]
            t0 = setup.tril[int(users[0])]
            one_cell = bool(np.all(setup.tril[users] == t0))
            order = _morton_order(setup.fw_positions[a0:a0 + n], t0) if n > 0 else np.zeros(0, int)
            P = setup.fw_positions[a0:a0 + n][order]
            pad = (-n) % 32
            starts[(a0, n)] = off
            pos_d.append(np.concatenate([P, np.repeat(P[-1:] if n else np.zeros((1, 3)), pad, 0)]))
            q_d.append(np.concatenate([setup.fw_charges[a0:a0 + n][order], np.zeros(pad)]))
            sp_d.append(np.concatenate([setup.fw_species[a0:a0 + n][order], np.zeros(pad, int)]))
            grp.append(_group_bounds(P, t0, one_cell, (n + pad) // 32))
            off += n + pad
        self.fw_pos = f32(np.concatenate([np.concatenate(pos_d), sp_bits(np.concatenate(sp_d))[:, None]], 1))
        self.fw_q = f32(np.concatenate(q_d))
        self.fw_group = f32(np.concatenate(grp).reshape(-1, 4)) if off > 0 else None
        self.fw_start = i32(np.array([starts[(a, n)] for a, n in zip(setup.fw_start.tolist(), setup.fw_count.tolist())]))
        self.fw_count = i32(setup.fw_count)
        self.guest = torch.zeros((s, setup.max_mol, apm, 4), dtype=torch.float32, device=dev)
        self.n_mol = torch.zeros(s, dtype=torch.int32, device=dev)
        # per guest molecule: its real-space energy with the rigid host and the key of the
        # positions it belongs to (kups_gcmc_args.host_cache); entries are keyed by positions,
        # so edits of the guests need no invalidation
        self.host_cache = torch.zeros((s, max(setup.max_mol, 1), 2), dtype=torch.float64, device=dev)
        # per-step U, N, U N, N^2, U^2 sums the kernel adds to (kups_gcmc_args.obs_sums)
        self.obs = torch.zeros((s, 5), dtype=torch.float64, device=dev)
        self.motif = f32(np.concatenate([setup.motif_positions, sp_bits(setup.motif_species)[:, None]], 1))
        self.motif_q = f32(setup.motif_charges)
        msc = np.bincount(setup.motif_species, minlength=T).astype(float)
        self.motif_sc = f64(msc)
        fwsc = np.stack([np.bincount(setup.fw_species[a:a + n], minlength=T) for a, n in
                         zip(setup.fw_start, setup.fw_count)]).astype(float)
        self.fw_sc = f64(fwsc)
        self.tril = f64(setup.tril)
        self.rc_lj, self.rc_ew, self.alpha = f64(setup.rc_lj), f64(setup.rc_ew), f64(setup.alpha)
        self.kn = i32(setup.kvec_n)
        nk = setup.kvec_n.shape[1]
        self.pk = f64(np.stack([prefactor(setup.tril[i], setup.kvec_n[i], setup.alpha[i]) for i in range(s)]))
        self.sk = torch.zeros((s, nk, 2), dtype=torch.float64, device=dev)
        # replicas of one cell share k vectors and P(k): the kernel then keeps one table for all
        self.k_shared = bool(s > 0 and (self.kn == self.kn[:1]).all().item() and (self.pk == self.pk[:1]).all().item())
        # kernel scratch: a reserved slab, float32 mirrors of S(k) and of (P(k), packed k)
        self.ws = torch.empty((3, s, max(nk, 1), 2), dtype=torch.float32, device=dev)
        self.lj_table = f32(np.stack([setup.sigma**2, 4 * setup.epsilon], -1).reshape(-1))
        vol = np.abs(setup.tril[:, 0] * setup.tril[:, 2] * setup.tril[:, 5])
        self.volume = vol
        self.tail = f64(np.stack([tail_coefficients(setup.sigma, setup.epsilon, setup.rc_lj[i], vol[i],
                                                    setup.tail_correction) for i in range(s)]))
        self.self_mol = f64(-TO_STANDARD_UNITS * setup.alpha / math.sqrt(math.pi) * float(np.sum(setup.motif_charges**2)))
        self.excl_mol = f64([exclusion_energy_of_molecule(setup.motif_positions, setup.motif_charges, a)
                             for a in setup.alpha])
        self.kT = f64(setup.temperature * BOLTZMANN_CONSTANT)
        self.log_activity = f64(setup.log_activity)
        self.energy = torch.zeros(s, dtype=torch.float64, device=dev)
        # framework-only structure factor (guests start empty)
        self._init_structure_factor()
        widths = np.tile(np.array([0.1, 0.1, 0.1, 0.1], np.float32), (s, 1))
        wmax = np.zeros((s, 4), np.float32)
        wmax[:, 0] = self._min_half_width()
        self.width, self.width_max = f32(widths), f32(wmax)
        self.history = torch.zeros((s, 4, 4), dtype=torch.int32, device=dev)
        self.history_index = torch.zeros((s, 4), dtype=torch.int32, device=dev)
        self.attempted = torch.zeros((s, 5), dtype=torch.int64, device=dev)
        self.accepted = torch.zeros((s, 5), dtype=torch.int64, device=dev)
        w = np.asarray(setup.move_weights, float)
        self.move_cum = np.cumsum(w[:3]) / w.sum()
        self.seed = seed
        self.step = 0
        self.status = new_status()
        self.proposal = None  # learned insertion density (LearnedInsertionProposal) or None: uniform
        self.block_threads = 0  # threads per CTA (0: library default); kups_gb300.autotune.autotune_gcmc picks one
        self.use_host_cache = True  # False: both ends of every move against the host, every step

    def _min_half_width(self):
        out = []
        for t in self.setup.tril:
            L = np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])
            v = abs(np.linalg.det(L))
            w = [v / np.linalg.norm(np.cross(L[1], L[2])), v / np.linalg.norm(np.cross(L[0], L[2])),
                 v / np.linalg.norm(np.cross(L[0], L[1]))]
            out.append(min(w) / 2)
        return np.array(out, np.float32)

    def _init_structure_factor(self):
        from .ewald import ewald_recip

        st = self.setup
        pos, q, off = [], [], [0]
        for a, n in zip(st.fw_start, st.fw_count):
            pos.append(st.fw_positions[a:a + n])
            q.append(st.fw_charges[a:a + n])
            off.append(off[-1] + n)
        P = torch.as_tensor(np.concatenate(pos), dtype=torch.float64, device="cuda")
        Q = torch.as_tensor(np.concatenate(q), dtype=torch.float64, device="cuda")
        O = torch.as_tensor(np.array(off, np.int32), device="cuda")
        _, _, _, sk, _ = ewald_recip(P, Q, O, int(np.max(st.fw_count)), self.tril, self.kn, self.alpha, grad_tril=False)
        self.sk.copy_(sk)

    def args(self, n_steps, proposals=None, out_delta=None, trace=None) -> _lib.GcmcArgs:
        a = _lib.GcmcArgs()
        st = self.setup
        a.fw_pos, a.fw_charge, a.fw_start, a.fw_count = (self.fw_pos.data_ptr(), self.fw_q.data_ptr(),
                                                         self.fw_start.data_ptr(), self.fw_count.data_ptr())
        a.guest_pos, a.n_mol = self.guest.data_ptr(), self.n_mol.data_ptr()
        a.motif_pos, a.motif_charge = self.motif.data_ptr(), self.motif_q.data_ptr()
        a.motif_species_count, a.fw_species_count = self.motif_sc.data_ptr(), self.fw_sc.data_ptr()
        a.tril, a.rc_lj, a.rc_ew, a.alpha = (self.tril.data_ptr(), self.rc_lj.data_ptr(), self.rc_ew.data_ptr(),
                                             self.alpha.data_ptr())
        a.kvec_n, a.prefactor, a.structure_factor = self.kn.data_ptr(), self.pk.data_ptr(), self.sk.data_ptr()
        a.lj_table, a.tail_coef = self.lj_table.data_ptr(), self.tail.data_ptr()
        a.self_energy_mol, a.exclusion_energy_mol = self.self_mol.data_ptr(), self.excl_mol.data_ptr()
        a.kT, a.log_activity, a.energy = self.kT.data_ptr(), self.log_activity.data_ptr(), self.energy.data_ptr()
        a.width, a.width_max = self.width.data_ptr(), self.width_max.data_ptr()
        a.history, a.history_index = self.history.data_ptr(), self.history_index.data_ptr()
        a.attempted, a.accepted = self.attempted.data_ptr(), self.accepted.data_ptr()
        a.proposals = proposals.data_ptr() if proposals is not None else None
        a.out_delta = out_delta.data_ptr() if out_delta is not None else None
        a.workspace = self.ws.data_ptr()
        a.fw_group = self.fw_group.data_ptr() if self.fw_group is not None else None
        a.obs_sums = self.obs.data_ptr()
        a.trace = trace.data_ptr() if trace is not None else None
        a.block_threads = int(self.block_threads)
        a.profile = self.profile.data_ptr() if getattr(self, "profile", None) is not None else None
        a.host_cache = self.host_cache.data_ptr() if self.use_host_cache else None
        a.k_shared = int(self.k_shared)
        if self.proposal is not None:
            a.proposal_node, a.proposal_cdf = self.proposal.node.data_ptr(), self.proposal.cdf.data_ptr()
            a.proposal_grid = self.proposal.grid
        for i in range(3):
            a.move_cum[i] = float(self.move_cum[i])
        a.coulomb_k = TO_STANDARD_UNITS
        a.seed, a.step0 = int(self.seed) & (2**64 - 1), int(self.step)
        a.n_systems, a.max_mol, a.atoms_per_mol = st.n_systems, st.max_mol, len(st.motif_charges)
        a.n_species, a.n_kvecs, a.n_steps, a.history_len = st.sigma.shape[0], st.kvec_n.shape[1], int(n_steps), 100
        return a

    def launch(self, n_steps, proposals=None, out_delta=None, trace=None):
        a = self.args(n_steps, proposals, out_delta, trace)
        rc = _lib.load().kups_gcmc_run(C.byref(a), self.status.data_ptr(), _stream())
        _lib.check(rc, "kups_gcmc_run")
        self.step += n_steps

    def run_traced(self, n_steps: int) -> np.ndarray:
        """n_steps steps of every system with the per-step record (``kups_gcmc_trace``): a
        structured array [n_steps, S] of the move kind, slot, decision, molecule count,
        energy change, ln acc, ln u, proposal log ratio, step width and proposed positions."""
        dt = np.dtype(_lib.GCMC_TRACE_DTYPE)
        buf = torch.zeros((n_steps * self.setup.n_systems * dt.itemsize,), dtype=torch.uint8, device="cuda")
        self.launch(n_steps, trace=buf)
        self.check()
        return buf.cpu().numpy().view(dt).reshape(n_steps, self.setup.n_systems)

    def __call__(self, key=None, n_steps: int = 1):
        """Propagator: n_steps MC steps of every system (one launch)."""
        if key is not None:
            from .md import key_to_seed

            self.seed = key_to_seed(key)
        self.launch(n_steps)
        return self

    def check(self):
        _lib.raise_status(read_status(self.status))

    def evaluate(self, kinds, mols, new_positions, force_reject=True):
        """One step with explicit proposals (no commit when force_reject): (dE, dE_real, dE_recip, log p) [S, 4]."""
        s = self.setup.n_systems
        apm = len(self.setup.motif_charges)
        props = np.zeros(s, dtype=[("kind", np.int32), ("mol", np.int32), ("force_reject", np.int32),
                                   ("pad", np.int32), ("pos", np.float32, (8, 4))])
        props["kind"], props["mol"], props["force_reject"] = kinds, mols, int(force_reject)
        sp = np.asarray(self.setup.motif_species, np.int32).view(np.float32)
        for i in range(s):
            if new_positions[i] is not None:
                props["pos"][i, :apm, :3] = new_positions[i]
                props["pos"][i, :apm, 3] = sp
        buf = torch.as_tensor(props.view(np.uint8).copy(), device="cuda")
        out = torch.zeros((s, 4), dtype=torch.float64, device="cuda")
        self.launch(1, proposals=buf, out_delta=out)
        return out.cpu().numpy()

    _STATE = ("guest", "n_mol", "sk", "energy", "width", "history", "history_index", "host_cache")

    def clone(self, seed: int | None = None) -> "GCMC":
        """A sampler on the same setup starting from this one's state (positions, counts,
        structure factors, energies, step widths); counters and statistics start at zero."""
        other = GCMC(self.setup, seed=self.seed if seed is None else seed)
        for k in self._STATE:
            getattr(other, k).copy_(getattr(self, k))
        other.step = self.step
        other.proposal = self.proposal
        other.block_threads = self.block_threads
        other.use_host_cache = self.use_host_cache
        return other

    def use_proposal(self, proposal):
        """Draw insertions from ``proposal``'s grid density (None: uniform, as the reference does)."""
        self.proposal = proposal

    def molecule_centres_frac(self) -> torch.Tensor:
        """Fractional coordinates in [0, 1) of every molecule's atom mean (atoms unwrapped against
        atom 0), all systems concatenated: the positions the learned proposal is trained on."""
        t = self.setup.tril  # host copy: the 3 x 3 inverses are formed with NumPy
        L = np.zeros((len(t), 3, 3))
        L[:, 0, 0], L[:, 1, 0], L[:, 1, 1], L[:, 2, 0], L[:, 2, 1], L[:, 2, 2] = np.asarray(t, np.float64).T
        inv = torch.as_tensor(np.linalg.inv(L), device="cuda")
        p = self.guest[..., :3].to(torch.float64)  # [S, M, apm, 3]
        f = torch.einsum("smai,sij->smaj", p, inv)
        d = f - f[:, :, :1]
        d = d - torch.round(d)
        c = f[:, :, 0] + d.mean(2)
        c = c - torch.floor(c)
        mask = torch.arange(p.shape[1], device=p.device)[None, :] < self.n_mol[:, None]
        return c[mask]

    def guest_positions(self) -> list[np.ndarray]:
        g = self.guest.cpu().numpy()
        n = self.n_mol.cpu().numpy()
        return [g[i, : n[i], :, :3].reshape(-1, 3) for i in range(len(n))]

    def set_guests(self, positions_per_system: list[np.ndarray]):
        """Place molecules (each [n_mol * apm, 3]) and update S(k) and counts (energy cache not changed)."""
        apm = len(self.setup.motif_charges)
        g = np.zeros(self.guest.shape, np.float32)
        sp = np.asarray(self.setup.motif_species, np.int32).view(np.float32)
        nm = []
        for i, p in enumerate(positions_per_system):
            m = len(p) // apm
            g[i, :m, :, :3] = np.asarray(p).reshape(m, apm, 3)
            g[i, :m, :, 3] = sp
            nm.append(m)
        self.guest.copy_(torch.as_tensor(g))
        self.n_mol.copy_(torch.as_tensor(np.array(nm, np.int32)))
        # structure factor of framework + guests
        from .ewald import ewald_recip

        st = self.setup
        pos, q, off = [], [], [0]
        for i, (a, n) in enumerate(zip(st.fw_start, st.fw_count)):
            gp = np.asarray(positions_per_system[i]).reshape(-1, 3)
            pos.append(np.concatenate([st.fw_positions[a:a + n], gp]))
            q.append(np.concatenate([st.fw_charges[a:a + n], np.tile(st.motif_charges, len(gp) // apm)]))
            off.append(off[-1] + len(pos[-1]))
        P = torch.as_tensor(np.concatenate(pos), dtype=torch.float64, device="cuda")
        Q = torch.as_tensor(np.concatenate(q), dtype=torch.float64, device="cuda")
        O = torch.as_tensor(np.array(off, np.int32), device="cuda")
        _, _, _, sk, _ = ewald_recip(P, Q, O, int(np.diff(off).max()), self.tril, self.kn, self.alpha, grad_tril=False)
        self.sk.copy_(sk)

    def run_blocks(self, n_blocks: int, block_steps: int) -> np.ndarray:
        """n_blocks launches of block_steps steps; returns the per-block sums of U, N, U N, N^2
        and U^2 of every system, [n_blocks, S, 5] float64, read back once at the end (the
        sums behind analyze_mcmc's per-step series, application/mcmc/analysis.py:82-158)."""
        out = torch.empty((n_blocks,) + tuple(self.obs.shape), dtype=torch.float64, device=self.obs.device)
        for b in range(n_blocks):
            self.obs.zero_()
            self.launch(block_steps)
            out[b].copy_(self.obs)
        self.check()
        return out.cpu().numpy()

    def analyze(self, block_sums, block_steps: int, n_blocks: int | None = None) -> dict:
        """Energy, loading and heat of adsorption (mean, SEM over blocks) per system from
        run_blocks' sums (analysis.gcmc_block_analysis)."""
        from .analysis import gcmc_block_analysis

        return gcmc_block_analysis(block_sums, block_steps, self.setup.temperature, n_blocks)

    def statistics(self):
        att = self.attempted.cpu().numpy()
        acc = self.accepted.cpu().numpy()
        return {m: (int(att[:, i].sum()), int(acc[:, i].sum())) for i, m in enumerate(MOVES)}

    # ------------------------------------------------------------------ stress of the guests
    def guest_table(self):
        """The guests as a particle table, grouped by system: positions f64 [A, 3] (the
        float32 state widened), charges, species, system and group (molecule index) [A]."""
        st = self.setup
        apm = len(st.motif_charges)
        keep = torch.arange(self.guest.shape[1], device="cuda")[None, :] < self.n_mol[:, None]
        pos = self.guest[..., :3][keep].reshape(-1, 3).to(torch.float64).contiguous()
        m = pos.shape[0] // apm
        sysi = torch.repeat_interleave(torch.arange(st.n_systems, device="cuda", dtype=torch.int32),
                                       (self.n_mol * apm).to(torch.int64))
        group = torch.repeat_interleave(torch.arange(m, device="cuda", dtype=torch.int32), apm)
        sp = torch.as_tensor(np.asarray(st.motif_species, np.int32), device="cuda").repeat(m)
        q = torch.as_tensor(np.asarray(st.motif_charges, np.float64), device="cuda").repeat(m)
        return pos, q, sp, sysi, group

    def guest_potential(self, positions, charges, species, system, group, tril=None):
        """Energy [S], dU/dx [A, 3] and dU/dtril [S, 6] of the guests alone (the guest-only
        state of mcmc_rigid.py:389-424): LJ and Ewald with each molecule's own pairs left out
        of the neighbour list, the excluded pairs' real-space minus vacuum Coulomb
        correction, and the LJ tail of the guest species counts (an energy c / V whose cell
        gradient is -U / L_aa on the diagonal)."""
        from .ewald import EwaldParameters, EwaldParticles, LJEwaldPotential
        from .potential import lennard_jones_tail_correction

        st = self.setup
        tr = torch.as_tensor(st.tril if tril is None else tril, dtype=torch.float64, device="cuda").reshape(-1, 6)
        apm = len(st.motif_charges)
        m = positions.shape[0] // apm
        a, b = np.nonzero(~np.eye(apm, dtype=bool))
        xe = (torch.arange(m, device="cuda", dtype=torch.int32)[:, None, None] * apm
              + torch.as_tensor(np.stack([a, b], 1), dtype=torch.int32, device="cuda")[None]).reshape(-1, 2)
        L = torch.zeros((tr.shape[0], 3, 3), dtype=torch.float64, device="cuda")
        L[:, [0, 1, 1, 2, 2, 2], [0, 0, 1, 0, 1, 2]] = tr
        frac = torch.einsum("ni,nij->nj", positions, torch.linalg.inv(L)[system.to(torch.int64)])
        xs = torch.round(frac[xe[:, 0].long()] - frac[xe[:, 1].long()]).to(torch.int32).contiguous()
        prm = EwaldParameters(torch.as_tensor(st.alpha), torch.as_tensor(st.rc_ew), torch.as_tensor(st.kvec_n))
        pot = LJEwaldPotential(prm, st.sigma, st.epsilon, st.rc_lj, exclusion_edges=(xe.contiguous(), xs))
        out = pot(EwaldParticles(positions, charges, system, species, exclusion=group), tr)
        energy, grad, gtril = out.total_energies, out.gradients.positions, out.gradients.unitcell
        if st.tail_correction and positions.shape[0]:
            et, _ = lennard_jones_tail_correction(species, system, tr, st.sigma, st.epsilon, st.rc_lj)
            dt = torch.zeros_like(gtril)
            dt[:, 0], dt[:, 2], dt[:, 5] = -et / tr[:, 0], -et / tr[:, 2], -et / tr[:, 5]
            energy, gtril = energy + et, gtril + dt
        return energy, grad, gtril

    def guest_stress(self) -> dict:
        """The rigid-MC app's stress record (``make_guest_stress``, mcmc_rigid.py:385-436;
        ``StressResult``, application/mcmc/data.py:170-175) for the current state, each
        [S, 3, 3] float64: ``potential`` the molecular virial stress (RASPA convention) of the
        guest-only energy and gradients; ``tail_correction`` P_tail I with P_tail of the full
        state (host and guests); ``ideal_gas`` N_mol k_B T / V I.  Their sum is the stress the
        reference's analysis block-averages (application/mcmc/analysis.py:186-190)."""
        from .observables import ideal_gas_pressure, virial_observables
        from .potential import lennard_jones_tail_correction

        st = self.setup
        S = st.n_systems
        pos, q, sp, sysi, group = self.guest_table()
        eye = torch.eye(3, dtype=torch.float64, device="cuda")
        if pos.shape[0]:
            _, grad, gtril = self.guest_potential(pos, q, sp, sysi, group)
            potential = virial_observables(pos, grad, sysi, st.tril, gtril, group=group,
                                           n_groups=pos.shape[0] // len(st.motif_charges),
                                           molecular=True)["molecular_stress"]
        else:
            potential = torch.zeros((S, 3, 3), dtype=torch.float64, device="cuda")
        if st.tail_correction:
            fw_sp = [np.asarray(st.fw_species[a:a + n]) for a, n in zip(st.fw_start, st.fw_count)]
            guests = sp.cpu().numpy()
            counts = (self.n_mol.cpu().numpy() * len(st.motif_charges)).tolist()
            offs = np.concatenate([[0], np.cumsum(counts)])
            full_sp = np.concatenate([np.concatenate([fw_sp[s], guests[offs[s]:offs[s + 1]]]) for s in range(S)])
            full_sys = np.concatenate([np.full(len(fw_sp[s]) + counts[s], s) for s in range(S)])
            _, p_tail = lennard_jones_tail_correction(full_sp, full_sys, st.tril, st.sigma, st.epsilon, st.rc_lj)
        else:
            p_tail = torch.zeros(S, dtype=torch.float64, device="cuda")
        p_ideal = ideal_gas_pressure(self.n_mol.to(torch.float64), st.temperature, st.tril)
        return {"potential": potential, "tail_correction": p_tail[:, None, None] * eye,
                "ideal_gas": p_ideal[:, None, None] * eye}
