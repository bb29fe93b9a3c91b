"""Per-system virial observables on the GPU: atomic and molecular virial stress,
lattice-gradient stress, kinetic energy and instantaneous pressure.

Mirrors src/kups/observables/stress.py (``stress_via_lattice_vector_gradients``,
``stress_via_virial_theorem``, ``molecular_stress_via_virial_theorem``, :123-190),
src/kups/observables/pressure.py (``pressure_from_stress``, ``ideal_gas_pressure``,
:27-61) and src/kups/md/observables.py (``instantaneous_pressure``, :38-61), on the
float64 particle table every other entry point uses: one ``kups_virial_stress`` call
evaluates all of them from positions, dU/dx, dU/dtril (and momenta) of any potential
(``kups_pair_edges``, ``kups_ewald_recip``, ``kups_bonded_edges``, ``LocalMLIAP``).
"""

from __future__ import annotations

import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status
from .units import BOLTZMANN_CONSTANT


def _f64(x):
    return torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()


def _i32(x):
    return torch.as_tensor(x, device="cuda").to(torch.int32).contiguous()


def virial_observables(positions, grad, system, tril, grad_tril=None, *, group=None, n_groups=None,
                       momenta=None, masses=None, molecular=False, check=True):
    """Every observable of one ``kups_virial_stress`` call as float64 device tensors:
    ``stress`` / ``lattice_stress`` (and ``molecular_stress`` when ``molecular``) [S, 3, 3],
    ``pressure`` [S] (2K / 3V + Tr(stress) / 3; K = 0 without momenta) and ``kinetic`` [S]
    when momenta are given.  ``group`` [N] assigns atoms to molecules for the molecular
    stress (``n_groups`` defaults to max + 1)."""
    lib = _lib.load()
    pos, g, sy, tr = _f64(positions), _f64(grad), _i32(system), _f64(tril)
    S, N = tr.shape[0], pos.shape[0]
    gt = _f64(grad_tril) if grad_tril is not None else None
    grp = _i32(group) if molecular else None
    if molecular:
        if group is None:
            raise ValueError("the molecular stress needs the group of every atom")
        n_groups = int(grp.max().item()) + 1 if n_groups is None and N else int(n_groups or 0)
    else:
        n_groups = 0
    mom = _f64(momenta) if momenta is not None else None
    ms = _f64(masses) if momenta is not None else None
    out = {"stress": torch.empty((S, 3, 3), dtype=torch.float64, device="cuda"),
           "lattice_stress": torch.empty((S, 3, 3), dtype=torch.float64, device="cuda"),
           "pressure": torch.empty(S, dtype=torch.float64, device="cuda")}
    if molecular:
        out["molecular_stress"] = torch.empty((S, 3, 3), dtype=torch.float64, device="cuda")
    if mom is not None:
        out["kinetic"] = torch.empty(S, dtype=torch.float64, device="cuda")
    ws_bytes = lib.kups_virial_stress_workspace_bytes(S, n_groups)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    status = new_status()
    ptr = lambda t: t.data_ptr() if t is not None else None
    rc = lib.kups_virial_stress(ptr(pos), ptr(g), ptr(sy), N, ptr(tr), ptr(gt), S, ptr(grp), n_groups, ptr(mom),
                                ptr(ms), ptr(out["stress"]), ptr(out.get("molecular_stress")),
                                ptr(out["lattice_stress"]), ptr(out.get("kinetic")), ptr(out["pressure"]),
                                ws.data_ptr(), ws_bytes, status.data_ptr(), _stream())
    _lib.check(rc, "kups_virial_stress")
    if check:
        _lib.raise_status(read_status(status))
    return out


def stress_via_virial_theorem(positions, grad, system, tril, grad_tril=None):
    """sigma = -(sum_i r_i (x) dU/dr_i + h^T dU/dh) / V per system [S, 3, 3] (stress.py:139-159)."""
    return virial_observables(positions, grad, system, tril, grad_tril)["stress"]


def molecular_stress_via_virial_theorem(positions, grad, system, group, tril, grad_tril=None, n_groups=None):
    """Molecular virial stress of the RASPA convention, symmetrised, [S, 3, 3]
    (stress.py:162-190); each system divided by its own volume."""
    return virial_observables(positions, grad, system, tril, grad_tril, group=group, n_groups=n_groups,
                              molecular=True)["molecular_stress"]


def stress_via_lattice_vector_gradients(tril, grad_tril):
    """sigma = -dU/dh / V per system [S, 3, 3] (stress.py:123-136)."""
    tr = _f64(tril)
    empty = torch.empty((0, 3), dtype=torch.float64, device="cuda")
    return virial_observables(empty, empty, torch.empty(0, dtype=torch.int32, device="cuda"), tr,
                              grad_tril)["lattice_stress"]


def pressure_from_stress(stress):
    """P = Tr(sigma) / 3 (pressure.py:27-29)."""
    return torch.diagonal(stress, dim1=-2, dim2=-1).sum(-1) / 3


def ideal_gas_pressure(counts, temperature, tril):
    """P = N k_B T / V per system (pressure.py:32-61); ``counts`` molecules (rigid-body MC)
    or atoms (MD)."""
    tr = _f64(tril)
    vol = (tr[:, 0] * tr[:, 2] * tr[:, 5]).abs()
    return _f64(counts) * BOLTZMANN_CONSTANT * _f64(temperature) / vol


def instantaneous_pressure(kinetic_energy, stress, tril):
    """P = 2K / 3V + Tr(sigma) / 3 (md/observables.py:38-61, d = 3)."""
    tr = _f64(tril)
    vol = (tr[:, 0] * tr[:, 2] * tr[:, 5]).abs()
    return 2.0 * _f64(kinetic_energy) / (3.0 * vol) + pressure_from_stress(stress)
