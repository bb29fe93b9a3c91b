"""Ewald summation on the GPU behind kUPS's Ewald potential interface.

Mirrors src/kups/potential/classical/ewald.py: ``EwaldParameters`` (:153-223,
alpha / real cutoff / integer ``reciprocal_lattice_shifts`` per system),
``estimate_ewald_parameters`` (:1166-1319) and ``kvecs_from_kmax``
(:1322-1339) as host-side setup (the reference also runs them on the host,
outside jit), and the energy terms (short range, long range, self, exclusion
correction) evaluated by the CUDA library: ``kups_pair_edges``,
``kups_ewald_recip`` and ``kups_ewald_self``.

``LJEwaldPotential`` is the summed LJ + Ewald potential of the ionic-melt
workload (real-space LJ and erfc Coulomb share one neighbour list) and
``LJEwaldMD`` integrates it with velocity Verlet or BAOAB, one step captured
in a CUDA graph and replayed.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .neighborlist import CellListNeighborList, NeighborListPoints, _f64, _i32, _stream, new_status, read_status
from .potential import PositionAndUnitCell, PotentialOut
from .units import BOLTZMANN_CONSTANT, TO_STANDARD_UNITS

TERM_LJ, TERM_EWALD_REAL, TERM_VACUUM = 1, 2, 4
TERM_ACCUMULATE = 8  # kups_lj_ewald_real_forces_packed: add onto energy / grad


# ----------------------------------------------------------------------------- host-side setup
def _lattice(tril):
    t = np.asarray(tril, dtype=np.float64)
    return np.array([[t[0], 0, 0], [t[1], t[2], 0], [t[3], t[4], t[5]]])


def kvecs_from_kmax(tril, kmax: float) -> np.ndarray:
    """Half-space integer k coefficients with |2 pi L^-1 n| <= kmax (ewald.py:1322-1339)."""
    inv = np.linalg.inv(_lattice(tril))
    rvecs = inv.T * 2 * np.pi
    min_length = np.min(np.linalg.svd(rvecs)[1])
    n = int(np.ceil(kmax / min_length))
    vecs = np.stack(np.meshgrid(np.arange(0, n + 1), np.arange(-n, n + 1), np.arange(-n, n + 1)), -1).reshape(-1, 3)
    return vecs[np.linalg.norm(vecs @ rvecs, axis=-1) <= kmax].astype(np.int32)


def kvecs_cube(kmax_int: int) -> np.ndarray:
    """Half-space integer box |n|_inf <= kmax_int, n_x >= 0 (the layout of kvecs_from_kmax)."""
    m = int(kmax_int)
    return np.stack(np.meshgrid(np.arange(0, m + 1), np.arange(-m, m + 1), np.arange(-m, m + 1)), -1).reshape(-1, 3).astype(np.int32)


def estimate_ewald_parameters(charges, tril, real_cutoff=None, alpha=None, epsilon_total=1e-8) -> dict:
    """Grid-search estimate of (alpha, rc, kmax) (ewald.py:1166-1319)."""
    from scipy import optimize, special

    q = np.asarray(charges, dtype=np.float64)
    t = np.asarray(tril, dtype=np.float64).reshape(6)
    L = _lattice(t)
    vol = abs(t[0] * t[2] * t[5])
    Q2, N = float(q @ q), q.size
    widths = vol / np.array([np.linalg.norm(np.cross(L[1], L[2])), np.linalg.norm(np.cross(L[0], L[2])),
                             np.linalg.norm(np.cross(L[0], L[1]))])
    max_radius = float(widths.min()) / 2
    eps = epsilon_total / 2
    length = vol ** (1 / 3)

    def grid_min(f, lo, hi, n=200):
        xs = np.linspace(lo, hi, n)
        return xs[np.argmin([f(x) for x in xs])]

    def e_real(rc, a):
        return np.inf if rc <= 0 or a <= 0 else (Q2 / np.sqrt(N)) * (special.erfc(a * rc) / rc)

    def e_recip(kc, a):
        if kc <= 0 or a <= 0:
            return np.inf
        x = -(kc**2) / (4 * a**2)
        return 0.0 if x < -700 else (Q2 * a / (np.sqrt(N) * np.pi)) * np.exp(x)

    def opt_rc(a):
        rc = grid_min(lambda r: abs(e_real(r, a) - eps), 0.01, min(20.0, max_radius)) if real_cutoff is None else real_cutoff
        return np.inf if e_real(rc, a) > 2 * eps else rc

    def opt_kc(a):
        kc = grid_min(lambda k: abs(e_recip(k, a) - eps), 0.1, 5.0)
        return np.inf if e_recip(kc, a) > 2 * eps else kc

    def cost(a):
        rc = opt_rc(a)
        if rc == np.inf:
            return np.inf
        kc = opt_kc(a)
        if kc == np.inf:
            return np.inf
        return float(rc**3 * N / vol * 4 / 3 * np.pi + (2 * kc * length / 2 / np.pi + 1) ** 3)

    if real_cutoff is not None:
        res = optimize.minimize_scalar(lambda z: abs(special.erfc(z) - real_cutoff * eps))
        if not res.success:
            raise ValueError("Failed to find alpha for given real space cutoff.")
        a = res.x / real_cutoff
        kmax = 2 * a * np.sqrt(-np.log(eps))
        return dict(alpha=a, real_cutoff=real_cutoff, k_max=kmax, error_real=e_real(real_cutoff, a),
                    error_recip=e_recip(kmax, a))
    a = grid_min(cost, 0.001, 2, 400) if alpha is None else alpha
    rc, kc = opt_rc(a), opt_kc(a)
    if rc <= 0 or kc <= 0 or rc == np.inf or kc == np.inf:
        raise ValueError("Invalid cutoff values computed")
    return dict(alpha=a, real_cutoff=rc, k_max=kc, error_real=e_real(rc, a), error_recip=e_recip(kc, a))


@dataclass
class EwaldParameters:
    alpha: torch.Tensor  # [S]
    cutoff: torch.Tensor  # [S]
    reciprocal_lattice_shifts: torch.Tensor  # int [S, n_k, 3], zero rows padding

    @classmethod
    def make(cls, charges, system, tril, epsilon_total=1e-8, real_cutoff=None) -> "EwaldParameters":
        """Per-system estimates, k lists zero-padded to the longest (ewald.py:170-223)."""
        q = np.asarray(charges, dtype=np.float64)
        sysi = np.asarray(system)
        tril = np.asarray(tril, dtype=np.float64).reshape(-1, 6)
        ests = [estimate_ewald_parameters(q[sysi == s], tril[s], real_cutoff, None, epsilon_total)
                for s in range(tril.shape[0])]
        ks = [kvecs_from_kmax(tril[s], e["k_max"]) for s, e in enumerate(ests)]
        nk = max(len(k) for k in ks)
        pad = np.stack([np.pad(k, [(0, nk - len(k)), (0, 0)]) for k in ks])
        return cls(torch.tensor([e["alpha"] for e in ests]), torch.tensor([e["real_cutoff"] for e in ests]),
                   torch.as_tensor(pad, dtype=torch.int32))


# ----------------------------------------------------------------------------- kernels
def _offsets(system: torch.Tensor, s: int) -> tuple[torch.Tensor, int]:
    counts = torch.bincount(system.long(), minlength=s)
    off = torch.zeros(s + 1, dtype=torch.int32, device="cuda")
    off[1:] = torch.cumsum(counts, 0).to(torch.int32)
    return off, int(counts.max()) if s > 0 else 0


class RecipWorkspace:
    def __init__(self):
        self.buf = None

    def get(self, nbytes):
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        return self.buf


def ewald_recip(positions, charges, sys_offset, max_atoms, tril, kvec_n, alpha, grad_tril=True, ws=None,
                out=None, status=None):
    """Reciprocal energy [S], dE/dx [N,3], dE/dtril [S,6], S(k) [S,nk,2] (atoms grouped by system).

    Every converted input is held in a local until the launch is enqueued, so
    no temporary's memory can be recycled under the kernel.
    """
    lib = _lib.load()
    pos, q, tril, al = _f64(positions), _f64(charges), _f64(tril), _f64(alpha)
    kn = _i32(kvec_n)
    off = _i32(sys_offset)
    s, nk = tril.shape[0], kn.shape[1]
    n = pos.shape[0]
    energy, grad, gtril, sk = out if out is not None else (
        torch.empty(s, dtype=torch.float64, device="cuda"), torch.empty((n, 3), dtype=torch.float64, device="cuda"),
        torch.empty((s, 6), dtype=torch.float64, device="cuda"), torch.empty((s, nk, 2), dtype=torch.float64, device="cuda"))
    nbytes = lib.kups_ewald_recip_workspace_bytes(s, nk)
    buf = (ws or RecipWorkspace()).get(nbytes)
    status = status if status is not None else new_status()
    rc = lib.kups_ewald_recip(pos.data_ptr(), q.data_ptr(), off.data_ptr(), s, int(max_atoms), tril.data_ptr(),
                              kn.data_ptr(), nk, al.data_ptr(), TO_STANDARD_UNITS, energy.data_ptr(),
                              grad.data_ptr(), gtril.data_ptr() if grad_tril else None, sk.data_ptr(), buf.data_ptr(),
                              buf.numel(), status.data_ptr(), _stream())
    _lib.check(rc, "kups_ewald_recip")
    return energy, grad, gtril, sk, status


def ewald_recip_energy(tril, kvec_n, alpha, structure_factor, ws=None, status=None):
    """K sum_k P(k) |S(k)|^2 per system from given structure factors (kups_ewald_recip_energy)."""
    lib = _lib.load()
    tril, al, sk = _f64(tril), _f64(alpha), _f64(structure_factor)
    kn = _i32(kvec_n)
    s, nk = tril.shape[0], kn.shape[1]
    energy = torch.empty(s, dtype=torch.float64, device="cuda")
    nbytes = lib.kups_ewald_recip_workspace_bytes(s, nk)
    buf = (ws or RecipWorkspace()).get(nbytes)
    status = status if status is not None else new_status()
    rc = lib.kups_ewald_recip_energy(tril.data_ptr(), kn.data_ptr(), nk, al.data_ptr(), s, TO_STANDARD_UNITS,
                                     sk.data_ptr(), energy.data_ptr(), buf.data_ptr(), buf.numel(), status.data_ptr(),
                                     _stream())
    _lib.check(rc, "kups_ewald_recip_energy")
    return energy


def ewald_self(charges, sys_offset, alpha, n_systems):
    lib = _lib.load()
    q, al, off = _f64(charges), _f64(alpha), _i32(sys_offset)
    e = torch.empty(n_systems, dtype=torch.float64, device="cuda")
    rc = lib.kups_ewald_self(q.data_ptr(), off.data_ptr(), n_systems, al.data_ptr(), TO_STANDARD_UNITS, e.data_ptr(),
                             _stream())
    _lib.check(rc, "kups_ewald_self")
    return e


def pair_edges(positions, system, species, charges, tril, edges, shifts, n_edges, terms, lj_sigma=None,
               lj_epsilon=None, lj_cutoff=None, alpha=None, ewald_cutoff=None, grad_tril=True, out=None, status=None):
    lib = _lib.load()
    pos, tril = _f64(positions), _f64(tril)
    n, s = pos.shape[0], tril.shape[0]
    keep = dict(system=_i32(system), edges=_i32(edges), shifts=_i32(shifts))
    for name, x, conv in (("species", species, _i32), ("charges", charges, _f64), ("sig", lj_sigma, _f64),
                          ("eps", lj_epsilon, _f64), ("rc_lj", lj_cutoff, _f64), ("alpha", alpha, _f64),
                          ("rc_ew", ewald_cutoff, _f64)):
        keep[name] = conv(torch.as_tensor(x)) if x is not None else None
    ptr = lambda k: keep[k].data_ptr() if keep[k] is not None else None
    energy, grad, gtril = out if out is not None else (
        torch.empty(s, dtype=torch.float64, device="cuda"), torch.empty((n, 3), dtype=torch.float64, device="cuda"),
        torch.empty((s, 6), dtype=torch.float64, device="cuda"))
    nsp = int(keep["sig"].shape[0]) if keep["sig"] is not None else 0
    status = status if status is not None else new_status()
    rc = lib.kups_pair_edges(pos.data_ptr(), ptr("system"), ptr("species"), ptr("charges"), n, tril.data_ptr(), s,
                             ptr("sig"), ptr("eps"), nsp, ptr("rc_lj"), ptr("alpha"), ptr("rc_ew"), TO_STANDARD_UNITS,
                             int(terms), ptr("edges"), ptr("shifts"), int(n_edges), energy.data_ptr(), grad.data_ptr(),
                             gtril.data_ptr() if grad_tril else None, status.data_ptr(), _stream())
    _lib.check(rc, "kups_pair_edges")
    return energy, grad, gtril


# ----------------------------------------------------------------------------- potentials
@dataclass
class EwaldParticles:
    positions: torch.Tensor  # f64 [N, 3], grouped by system
    charges: torch.Tensor
    system: torch.Tensor
    species: torch.Tensor | None = None
    exclusion: torch.Tensor | None = None


@dataclass
class LJEwaldCache:
    """What a patched call starts from: the total energies and the structure factors S(k) of the
    current state (``EwaldCache``, src/kups/potential/classical/ewald.py:86-120)."""

    total_energies: torch.Tensor  # [S]
    structure_factor: torch.Tensor  # [S, n_k, 2]


class LJEwaldPotential:
    """E = LJ (optional) + Ewald (short range + long range + self - excluded vacuum Coulomb).

    With a ``patch`` (particles moved to new positions) the energies after the patch come from
    the cache of the current state: the real-space terms of the removed and added edges of
    ``neighborlist_changes`` (``LocalGraphSumComposer``, src/kups/potential/common/graph.py:419-453),
    the intramolecular correction at the old and new positions, and the long-range energy of
    S(k) + delta S(k) with delta S(k) the moved particles' old copies (charge -q) and new
    positions (+q) (``_structure_factor_update``, ewald.py:442-486; ``EwaldLongRangeComposer``,
    :604-657); no gradients.  The returned cache holds the patched energies and S(k), to be
    kept if the move is accepted.
    """

    def __init__(self, ewald: EwaldParameters, lj_sigma=None, lj_epsilon=None, lj_cutoff=None,
                 neighborlist: CellListNeighborList | None = None, exclusion_edges=None):
        self.ewald = ewald
        self.lj = (lj_sigma, lj_epsilon, lj_cutoff) if lj_sigma is not None else None
        self.neighborlist = neighborlist or CellListNeighborList(avg_edges=512)
        self.exclusion_edges = exclusion_edges  # (edges [E,2], shifts [E,3]) intramolecular pairs
        self.ws = RecipWorkspace()

    def __call__(self, particles: EwaldParticles, tril, patch=None, cache: LJEwaldCache | None = None) -> PotentialOut:
        tril = _f64(tril)
        s = tril.shape[0]
        alpha, rc_ew = _f64(self.ewald.alpha), _f64(self.ewald.cutoff)
        rc_nl = rc_ew.clone()
        terms = TERM_EWALD_REAL
        sig = eps = rc_lj = None
        if self.lj is not None:
            sig, eps, rc_lj = (_f64(torch.as_tensor(x)) for x in self.lj)
            rc_lj = rc_lj.reshape(-1).expand(s).contiguous()
            rc_nl = torch.maximum(rc_nl, rc_lj)
            terms |= TERM_LJ
        if patch is not None:
            return self._patched(particles, tril, patch, cache, terms, sig, eps, rc_lj, alpha, rc_ew, rc_nl)
        pts = NeighborListPoints(particles.positions, particles.system, None, particles.exclusion)
        e, self.neighborlist = self.neighborlist.call_and_fix(pts, None, tril, rc_nl)
        en, g, gt = pair_edges(particles.positions, particles.system, particles.species, particles.charges, tril,
                               e.indices, e.shifts.view(-1, 3), e.n_edges, terms, sig, eps, rc_lj, alpha, rc_ew)
        off, mx = _offsets(_i32(particles.system), s)
        self._last_recip = ewald_recip(particles.positions, particles.charges, off, mx, tril,
                                       self.ewald.reciprocal_lattice_shifts, alpha, ws=self.ws)
        el, gl, gtl, _, _ = self._last_recip
        es = ewald_self(particles.charges, off, alpha, s)
        energy, grad, gtril = en + el + es, g + gl, gt + gtl
        if self.exclusion_edges is not None:
            xe, xs = self.exclusion_edges
            ex, gx, gtx = pair_edges(particles.positions, particles.system, None, particles.charges, tril, xe, xs,
                                     xe.shape[0], TERM_EWALD_REAL | TERM_VACUUM, alpha=alpha,
                                     ewald_cutoff=torch.full_like(rc_ew, float("inf")))
            energy, grad, gtril = energy + ex, grad + gx, gtril + gtx
        _, _, _, sk, _ = self._last_recip
        return PotentialOut(energy, PositionAndUnitCell(grad, gtril), cache=LJEwaldCache(energy, sk))

    def _patched(self, particles, tril, patch, cache, terms, sig, eps, rc_lj, alpha, rc_ew, rc_nl) -> PotentialOut:
        from .potential import changed_edges, patched_positions

        if cache is None:
            cache = self(particles, tril).cache
        s = tril.shape[0]
        added, removed = changed_edges(self.neighborlist, particles.positions, particles.system, None,
                                       particles.exclusion, tril, rc_nl, patch)
        old = _f64(particles.positions)
        new = patched_positions(old, patch)
        pe = lambda pos, e: pair_edges(pos, particles.system, particles.species, particles.charges, tril, e.indices,
                                       e.shifts.view(-1, 3), e.n_edges, terms, sig, eps, rc_lj, alpha, rc_ew,
                                       grad_tril=False)[0]
        de = pe(new, added) - pe(old, removed)
        if self.exclusion_edges is not None:
            xe, xs = self.exclusion_edges
            inf = torch.full_like(rc_ew, float("inf"))
            ex = lambda pos: pair_edges(pos, particles.system, None, particles.charges, tril, xe, xs, xe.shape[0],
                                        TERM_EWALD_REAL | TERM_VACUUM, alpha=alpha, ewald_cutoff=inf,
                                        grad_tril=False)[0]
            de = de + ex(new) - ex(old)
        # S(k) change: the moved particles' old copies with -q and new positions with +q, by system
        idx = _i32(patch.indices).long()
        q = _f64(particles.charges)[idx]
        sysm = _i32(particles.system)[idx]
        both_sys = torch.cat([sysm, sysm])
        order = torch.argsort(both_sys, stable=True)
        pos_m = torch.cat([old[idx], new[idx]])[order].contiguous()
        q_m = torch.cat([-q, q])[order].contiguous()
        off_m, mx = _offsets(both_sys[order], s)
        _, _, _, dsk, _ = ewald_recip(pos_m, q_m, off_m, mx, tril, self.ewald.reciprocal_lattice_shifts, alpha,
                                      grad_tril=False, ws=self.ws)
        sk_new = cache.structure_factor + dsk
        kn = self.ewald.reciprocal_lattice_shifts
        de = de + ewald_recip_energy(tril, kn, alpha, sk_new, ws=self.ws) - ewald_recip_energy(
            tril, kn, alpha, cache.structure_factor, ws=self.ws)
        e_new = cache.total_energies + de
        return PotentialOut(e_new, None, None, cache=LJEwaldCache(e_new, sk_new))


# ----------------------------------------------------------------------------- MD
def _perpendicular_widths(tril) -> np.ndarray:
    """[S, 3] distances between opposite faces of each lower-triangular cell (host, float64)."""
    t = np.asarray(torch.as_tensor(tril).detach().cpu().numpy(), np.float64).reshape(-1, 6)
    L = np.zeros((len(t), 3, 3))
    L[:, 0, 0], L[:, 1, 0], L[:, 1, 1], L[:, 2, 0], L[:, 2, 1], L[:, 2, 2] = t.T
    vol = np.abs(L[:, 0, 0] * L[:, 1, 1] * L[:, 2, 2])
    cross = lambda a, b: np.linalg.norm(np.cross(L[:, a], L[:, b]), axis=1)
    return np.stack([vol / cross(1, 2), vol / cross(2, 0), vol / cross(0, 1)], 1)


class LJEwaldMD:
    """VV (NVE) or BAOAB steps of LJ + Ewald dynamics on the float64 particle table.

    One step = kick / drift (/ thermostat / drift) / neighbour list / real-space
    pairs / reciprocal space / self / kick, all stream-ordered with no host
    synchronisation (the edge list is passed at capacity; padded rows are
    skipped in the kernel), so a step is captured once in a CUDA graph and
    replayed.  Real space: when every cell width is at least twice the cutoff
    (every pair within it is its minimum image) all pairs of a system are
    evaluated from shared-memory tiles with no stored list
    (kups_lj_ewald_real_forces); otherwise the neighbour list is rebuilt every
    step, as the reference MD application does, and the edges are evaluated by
    kups_pair_edges in float64.  ``real_space`` forces one of the two ("allpairs",
    "edges"; "auto" picks all pairs when it applies).
    """

    def __init__(self, particles: EwaldParticles, masses, tril, ewald: EwaldParameters, time_step, lj_sigma=None,
                 lj_epsilon=None, lj_cutoff=None, integrator="velocity_verlet", temperature=None, friction=None,
                 avg_edges=None, seed=0, real_space="auto"):
        self.p = particles
        self.n = particles.positions.shape[0]
        self.tril = _f64(tril)
        self.s = self.tril.shape[0]
        self.masses = _f64(masses)
        self.system = _i32(particles.system)
        self.species = _i32(particles.species) if particles.species is not None else torch.zeros(self.n, dtype=torch.int32, device="cuda")
        self.q = _f64(particles.charges)
        self.dt = _f64(torch.as_tensor(time_step, dtype=torch.float64).reshape(-1).expand(self.s))
        self.integrator = integrator
        self.kT = _f64(torch.as_tensor(temperature if temperature is not None else 0.0, dtype=torch.float64).reshape(-1).expand(self.s) * BOLTZMANN_CONSTANT)
        self.friction = _f64(torch.as_tensor(friction if friction is not None else 0.0, dtype=torch.float64).reshape(-1).expand(self.s))
        self.alpha, self.rc_ew = _f64(ewald.alpha), _f64(ewald.cutoff)
        self.kn = _i32(ewald.reciprocal_lattice_shifts)
        self.lj = lj_sigma is not None
        if self.lj:
            self.sig, self.eps = _f64(torch.as_tensor(lj_sigma)), _f64(torch.as_tensor(lj_epsilon))
            self.rc_lj = _f64(torch.as_tensor(lj_cutoff, dtype=torch.float64).reshape(-1).expand(self.s))
            self.rc_nl = torch.maximum(self.rc_ew, self.rc_lj)
        else:
            self.sig = self.eps = self.rc_lj = None
            self.rc_nl = self.rc_ew.clone()
        self.off, self.max_atoms = _offsets(self.system, self.s)
        vol = float((self.tril[:, 0] * self.tril[:, 2] * self.tril[:, 5]).abs().min())
        nsp = int(self.sig.shape[0]) if self.lj else 1
        grouped = bool((self.system[1:] >= self.system[:-1]).all()) if self.n > 1 else True
        fits = grouped and nsp <= 8 and bool(
            (_perpendicular_widths(self.tril).min(1) >= 2.0 * self.rc_nl.cpu().numpy()).all())
        if real_space not in ("auto", "allpairs", "edges"):
            raise ValueError("real_space is 'auto', 'allpairs' or 'edges'")
        if real_space == "allpairs" and not fits:
            raise ValueError("the all-pairs real space needs systems grouped in order, at most 8 species and "
                             "every cell width at least twice the cutoff")
        # all pairs in float32 (no stored list) when it applies, else the float64 edge path
        self.allpairs = fits and real_space != "edges"
        if avg_edges is None:
            avg_edges = int(4 / 3 * math.pi * float(self.rc_nl.max()) ** 3 * self.n / vol * 1.5) + 64
        self.cap = avg_edges * self.n
        self.edges = torch.empty((self.cap, 2), dtype=torch.int32, device="cuda")
        self.shifts = torch.empty((self.cap, 3), dtype=torch.int32, device="cuda")
        self.n_edges = torch.zeros(1, dtype=torch.int64, device="cuda")
        lib = _lib.load()
        self.nl_ws = torch.empty(lib.kups_neighborlist_workspace_bytes(self.n, self.s), dtype=torch.uint8, device="cuda")
        self.real_ws = torch.empty(lib.kups_lj_ewald_real_forces_workspace_bytes(self.s, self.max_atoms),
                                   dtype=torch.uint8, device="cuda") if self.allpairs else None
        self.rws = RecipWorkspace()
        self.rws.get(lib.kups_ewald_recip_workspace_bytes(self.s, self.kn.shape[1]))
        self.status = new_status()
        f64 = dict(dtype=torch.float64, device="cuda")
        self.e_pair, self.g_pair, self.t_pair = torch.empty(self.s, **f64), torch.empty((self.n, 3), **f64), torch.empty((self.s, 6), **f64)
        self.e_rec, self.g_rec, self.t_rec = torch.empty(self.s, **f64), torch.empty((self.n, 3), **f64), torch.empty((self.s, 6), **f64)
        self.sk = torch.empty((self.s, self.kn.shape[1], 2), **f64)
        self.grad = torch.zeros((self.n, 3), **f64)
        self.energy = torch.zeros(self.s, **f64)
        self.e_self = ewald_self(self.q, self.off, self.alpha, self.s)
        self.incl = self.system
        self.excl = torch.arange(self.n, dtype=torch.int32, device="cuda")
        self.seed = seed
        self.step_counter = torch.zeros(1, dtype=torch.int64)
        # the Langevin noise counter of the captured BAOAB step lives on the device
        self.counter = torch.zeros(1, dtype=torch.int64, device="cuda")
        # partner shares per 16-atom block of the all-pairs real space (0: the library default of
        # one; autotune.autotune_lj_ewald picks one per workload)
        self.real_splits = 0
        self.graph = None

    def _forces(self):
        lib = _lib.load()
        pos = self.p.positions
        if self.allpairs:
            terms = TERM_EWALD_REAL | (TERM_LJ if self.lj else 0)
            nsp = int(self.sig.shape[0]) if self.lj else 1
            # reciprocal space writes energy and grad; real space adds onto them
            ewald_recip(pos, self.q, self.off, self.max_atoms, self.tril, self.kn, self.alpha, grad_tril=False,
                        ws=self.rws, out=(self.energy, self.grad, self.t_rec, self.sk), status=self.status)
            rc = lib.kups_lj_ewald_real_forces_packed(
                pos.data_ptr(), self.q.data_ptr(), self.species.data_ptr(), self.off.data_ptr(), self.s,
                self.max_atoms, self.tril.data_ptr(), self.sig.data_ptr() if self.lj else None,
                self.eps.data_ptr() if self.lj else None, nsp, self.rc_lj.data_ptr() if self.lj else None,
                self.alpha.data_ptr(), self.rc_ew.data_ptr(), TO_STANDARD_UNITS,
                terms | TERM_ACCUMULATE | (self.real_splits << 8),
                self.energy.data_ptr(), self.grad.data_ptr(), self.real_ws.data_ptr(), self.real_ws.numel(),
                self.status.data_ptr(), _stream())
            _lib.check(rc, "kups_lj_ewald_real_forces_packed")
            self.energy.add_(self.e_self)
            return
        rc = lib.kups_neighborlist_build(pos.data_ptr(), self.system.data_ptr(), self.incl.data_ptr(),
                                         self.excl.data_ptr(), self.n, self.s, self.tril.data_ptr(),
                                         self.rc_nl.data_ptr(), self.s, self.edges.data_ptr(), self.shifts.data_ptr(),
                                         self.cap, self.n_edges.data_ptr(), self.nl_ws.data_ptr(), self.nl_ws.numel(),
                                         self.status.data_ptr(), _stream())
        _lib.check(rc, "kups_neighborlist_build")
        terms = TERM_EWALD_REAL | (TERM_LJ if self.lj else 0)
        pair_edges(pos, self.system, self.species, self.q, self.tril, self.edges, self.shifts, self.cap, terms,
                   self.sig, self.eps, self.rc_lj, self.alpha, self.rc_ew, grad_tril=False,
                   out=(self.e_pair, self.g_pair, self.t_pair), status=self.status)
        ewald_recip(pos, self.q, self.off, self.max_atoms, self.tril, self.kn, self.alpha, grad_tril=False,
                    ws=self.rws, out=(self.e_rec, self.g_rec, self.t_rec, self.sk), status=self.status)
        torch.add(self.g_pair, self.g_rec, out=self.grad)
        torch.add(self.e_pair, self.e_rec, out=self.energy)
        self.energy.add_(self.e_self)

    def _step(self, step):
        lib = _lib.load()
        st = _stream()
        p = self.p
        lib.kups_md_kick(p_mom := self.mom.data_ptr(), self.grad.data_ptr(), self.system.data_ptr(),
                         self.dt.data_ptr(), 0.5, self.n, st)
        if self.integrator == "baoab":
            lib.kups_md_drift(p.positions.data_ptr(), p_mom, self.masses.data_ptr(), self.system.data_ptr(),
                              self.dt.data_ptr(), self.tril.data_ptr(), 0.5, self.n, st)
            lib.kups_md_thermostat_counted(p_mom, self.masses.data_ptr(), self.system.data_ptr(),
                                           self.dt.data_ptr(), self.kT.data_ptr(), self.friction.data_ptr(),
                                           self.seed, self.counter.data_ptr(), self.n, st)
            self.counter.add_(1)
            lib.kups_md_drift(p.positions.data_ptr(), p_mom, self.masses.data_ptr(), self.system.data_ptr(),
                              self.dt.data_ptr(), self.tril.data_ptr(), 0.5, self.n, st)
        else:
            lib.kups_md_drift(p.positions.data_ptr(), p_mom, self.masses.data_ptr(), self.system.data_ptr(),
                              self.dt.data_ptr(), self.tril.data_ptr(), 1.0, self.n, st)
        self._forces()
        lib.kups_md_kick(p_mom, self.grad.data_ptr(), self.system.data_ptr(), self.dt.data_ptr(), 0.5, self.n, st)

    def start(self, momenta):
        self.mom = _f64(momenta).clone()
        self.p.positions = _f64(self.p.positions).clone()
        self._forces()
        torch.cuda.synchronize()

    def run(self, n_steps: int, use_graph: bool = True):
        """n_steps steps; the Langevin counter (on the device, so that a replayed graph advances
        it) goes up by one per step."""
        if not use_graph:
            for _ in range(n_steps):
                self._step(int(self.step_counter.item()))
                self.step_counter += 1
            return
        if self.graph is None:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._step(0)  # warm-up outside capture
            torch.cuda.current_stream().wait_stream(s)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                self._step(0)
            n_steps -= 1  # the warm-up advanced the state; capture only records
        for _ in range(max(n_steps, 0)):
            self.graph.replay()

    def check(self):
        _lib.raise_status(read_status(self.status))

    def kinetic_energy(self):
        ke = 0.5 * (self.mom**2).sum(-1) / self.masses
        return torch.zeros(self.s, dtype=torch.float64, device="cuda").index_add_(0, self.system.long(), ke)
