"""ctypes binding of the kups_gb300 C ABI (``include/kups_gb300.h``).

The library is the only compute path of this package: if it cannot be loaded
the calls raise instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkups_gb300.so")

KUPS_OK = 0
KUPS_ERR_CAPACITY = 1
KUPS_ERR_NONFINITE = 2
KUPS_ERR_INVALID = 3
KUPS_ERR_CUDA = 4
KUPS_ERR_UNSUPPORTED = 5

KUPS_CAP_EDGES = 1
KUPS_CAP_NEIGHBORS = 2
KUPS_CAP_GHOSTS = 3
KUPS_CAP_CELLS = 4
KUPS_CAP_ATOMS = 5

CAPACITY_NAMES = {1: "edges", 2: "neighbors", 3: "ghosts", 4: "cells", 5: "atoms"}


class Status(C.Structure):
    _fields_ = [("code", C.c_int32), ("detail", C.c_int32), ("required", C.c_int64), ("first_bad", C.c_int64)]


class MdArgs(C.Structure):
    _fields_ = [
        ("pos", C.c_void_p), ("mom", C.c_void_p), ("force", C.c_void_p),
        ("sys_offset", C.c_void_p), ("order", C.c_void_p), ("tril", C.c_void_p),
        ("cutoff", C.c_void_p), ("skin", C.c_void_p), ("dt", C.c_void_p), ("kT", C.c_void_p),
        ("friction", C.c_void_p), ("lj_table", C.c_void_p),
        ("energy", C.c_void_p), ("kinetic", C.c_void_p), ("virial", C.c_void_p), ("pressure", C.c_void_p),
        ("trace_pe", C.c_void_p), ("trace_ke", C.c_void_p), ("rebuilds", C.c_void_p), ("profile", C.c_void_p),
        ("n_atoms", C.c_int64), ("n_systems", C.c_int32), ("n_species", C.c_int32),
        ("n_steps", C.c_int32), ("integrator", C.c_int32), ("forces_valid", C.c_int32),
        ("neighbor_capacity", C.c_int32), ("seed", C.c_uint64), ("step0", C.c_uint64),
        ("n_ctas", C.c_int32), ("block_threads", C.c_int32),
        ("min_lanes_per_atom", C.c_int32), ("reuse_lists", C.c_int32),
        ("thermostat_tau", C.c_void_p), ("target_pressure", C.c_void_p), ("barostat_tau", C.c_void_p),
        ("compressibility", C.c_void_p), ("min_scale", C.c_void_p), ("cell", C.c_void_p),
        ("trace_virial", C.c_void_p), ("atom_base", C.c_int64), ("system_base", C.c_int32),
        ("pad_base", C.c_int32),
    ]


class GcmcProposal(C.Structure):
    _fields_ = [("kind", C.c_int32), ("mol", C.c_int32), ("force_reject", C.c_int32), ("pad", C.c_int32),
                ("pos", (C.c_float * 4) * 8)]


class GcmcArgs(C.Structure):
    _fields_ = [
        ("fw_pos", C.c_void_p), ("fw_charge", C.c_void_p), ("fw_start", C.c_void_p), ("fw_count", C.c_void_p),
        ("guest_pos", C.c_void_p), ("n_mol", C.c_void_p), ("motif_pos", C.c_void_p), ("motif_charge", C.c_void_p),
        ("motif_species_count", C.c_void_p), ("fw_species_count", C.c_void_p), ("tril", C.c_void_p),
        ("rc_lj", C.c_void_p), ("rc_ew", C.c_void_p), ("alpha", C.c_void_p), ("kvec_n", C.c_void_p),
        ("prefactor", C.c_void_p), ("structure_factor", C.c_void_p), ("lj_table", C.c_void_p),
        ("tail_coef", C.c_void_p), ("self_energy_mol", C.c_void_p), ("exclusion_energy_mol", C.c_void_p),
        ("kT", C.c_void_p), ("log_activity", C.c_void_p), ("energy", C.c_void_p), ("width", C.c_void_p),
        ("width_max", C.c_void_p), ("history", C.c_void_p), ("history_index", C.c_void_p),
        ("attempted", C.c_void_p), ("accepted", C.c_void_p), ("proposals", C.c_void_p), ("out_delta", C.c_void_p),
        ("proposal_node", C.c_void_p), ("proposal_cdf", C.c_void_p), ("workspace", C.c_void_p),
        ("fw_group", C.c_void_p), ("obs_sums", C.c_void_p),
        ("move_cum", C.c_float * 3), ("pad0", C.c_float), ("coulomb_k", C.c_double), ("seed", C.c_uint64),
        ("step0", C.c_uint64), ("n_systems", C.c_int32), ("max_mol", C.c_int32), ("atoms_per_mol", C.c_int32),
        ("n_species", C.c_int32), ("n_kvecs", C.c_int32), ("n_steps", C.c_int32), ("history_len", C.c_int32),
        ("proposal_grid", C.c_int32), ("trace", C.c_void_p), ("block_threads", C.c_int32), ("pad1", C.c_int32),
        ("profile", C.c_void_p), ("host_cache", C.c_void_p), ("k_shared", C.c_int32), ("pad2", C.c_int32),
    ]


# numpy layout of kups_gcmc_trace (one record per step and system)
GCMC_TRACE_DTYPE = [("kind", "<i4"), ("mol", "<i4"), ("accept", "<i4"), ("n_mol", "<i4"), ("has_old", "<i4"),
                    ("has_new", "<i4"), ("width", "<f4"), ("pad", "<i4"), ("de", "<f8"), ("log_p", "<f8"),
                    ("log_u", "<f8"), ("ln_ratio", "<f8"), ("new_pos", "<f4", (8, 4))]


class Mlp(C.Structure):
    _fields_ = [("param", C.c_void_p), ("param_bf16", C.c_void_p), ("grad", C.c_void_p), ("adam_m", C.c_void_p),
                ("adam_v", C.c_void_p), ("freq", C.c_void_p), ("param_bf16_t", C.c_void_p)]


# Every symbol declared in include/kups_gb300.h: name -> (restype, argtypes)
_P, _I32, _I64, _SZ = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
SIGNATURES = {
    "kups_version": (C.c_char_p, []),
    "kups_error_string": (C.c_char_p, [_I32]),
    "kups_neighborlist_workspace_bytes": (_SZ, [_I64, _I32]),
    "kups_neighborlist_build": (_I32, [_P, _P, _P, _P, _I64, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P, _SZ, _P, _P]),
    "kups_neighborlist_rh_workspace_bytes": (_SZ, [_I64, _I64, _I32]),
    "kups_neighborlist_build_rh": (_I32, [_P, _P, _P, _P, _I64, _P, _P, _P, _P, _I64, _P, _I32, _P, _P, _I32, _P, _P,
                                          _I64, _P, _P, _SZ, _P, _P]),
    "kups_neighborlist_split_workspace_bytes": (_SZ, [_I64, _I64]),
    "kups_neighborlist_split_changes": (_I32, [_P, _P, _P, _I64, _I64, _P, _I64, _P, _P, _I64, _P, _P, _P, _I64, _P,
                                               _P, _SZ, _P, _P]),
    "kups_edge_vectors": (_I32, [_P, _P, _I64, _P, _I32, _P, _P, _I64, _P, _P]),
    "kups_edge_segment_sum": (_I32, [_P, _I32, _P, _I64, _I64, _P, _P]),
    "kups_edge_gradients": (_I32, [_P, _P, _I64, _I32, _P, _P, _I64, _P, _P, _P]),
    "kups_lj_edges": (_I32, [_P, _P, _P, _I64, _P, _P, _I32, _P, _P, _I32, _P, _P, _I64, _P, _P, _P, _I32, _P, _P]),
    "kups_lj_md_workspace_bytes": (_SZ, [C.POINTER(MdArgs)]),
    "kups_lj_md_run": (_I32, [C.POINTER(MdArgs), _P, _SZ, _P, _P]),
    "kups_lj_md_max_atoms": (_I32, []),
    "kups_md_pack": (_I32, [_P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "kups_md_unpack": (_I32, [_P, _P, _P, _P, _I64, _P, _P, _P, _P]),
    "kups_ewald_recip_workspace_bytes": (_SZ, [_I32, _I32]),
    "kups_ewald_recip": (_I32, [_P, _P, _P, _I32, _I32, _P, _P, _I32, _P, C.c_double, _P, _P, _P, _P, _P, _SZ, _P, _P]),
    "kups_ewald_recip_energy": (_I32, [_P, _P, _I32, _P, _I32, C.c_double, _P, _P, _P, _SZ, _P, _P]),
    "kups_ewald_recip_static": (_I32, [_P, _P, _P, _I32, _I32, _P, _P, _I32, _P, C.c_double, _P, _P, _P, _P, _P, _P]),
    "kups_lj_ewald_real_forces": (_I32, [_P, _P, _P, _P, _I32, _I32, _P, _P, _P, _I32, _P, _P, _P, C.c_double, _I32, _P, _P, _P, _P]),
    "kups_lj_ewald_real_forces_workspace_bytes": (C.c_size_t, [_I32, _I32]),
    "kups_lj_ewald_real_forces_packed": (_I32, [_P, _P, _P, _P, _I32, _I32, _P, _P, _P, _I32, _P, _P, _P, C.c_double, _I32, _P, _P, _P, C.c_size_t, _P, _P]),
    "kups_ewald_self": (_I32, [_P, _P, _I32, _P, C.c_double, _P, _P]),
    "kups_md_kick": (_I32, [_P, _P, _P, _P, C.c_double, _I64, _P]),
    "kups_md_drift": (_I32, [_P, _P, _P, _P, _P, _P, C.c_double, _I64, _P]),
    "kups_md_thermostat": (_I32, [_P, _P, _P, _P, _P, _P, C.c_uint64, C.c_uint64, _I64, _P]),
    "kups_md_thermostat_counted": (_I32, [_P, _P, _P, _P, _P, _P, C.c_uint64, _P, _I64, _P]),
    "kups_virial_stress_workspace_bytes": (C.c_size_t, [_I32, _I32]),
    "kups_virial_stress": (_I32, [_P, _P, _P, _I64, _P, _P, _I32, _P, _I32, _P, _P, _P, _P, _P, _P, _P, _P,
                                  C.c_size_t, _P, _P]),
    "kups_gcmc_run": (_I32, [C.POINTER(GcmcArgs), _P, _P]),
    "kups_mlp_workspace_bytes": (_SZ, [_I64]),
    "kups_mlp_init": (_I32, [_P, C.c_uint64, _P]),
    "kups_mlp_fwd": (_I32, [_P, _P, _I64, _P, _P, _SZ, _P, _P]),
    "kups_mlp_nce_batch": (_I32, [_P, _I64, _I32, C.c_uint64, C.c_uint64, _P, _P, _P]),
    "kups_mlp_bwd": (_I32, [_P, _P, _P, _I32, _P, _P, _SZ, _P, _P]),
    "kups_mlp_adam": (_I32, [_P, _I64, C.c_float, C.c_float, C.c_float, C.c_float, _P]),
    "kups_mlp_grid_norm": (_I32, [_P, _I32, C.c_float, C.c_float, _P, _P, _P, _SZ, _P, _P]),
    "kups_proposal_sample": (_I32, [_P, _P, _I32, _I64, C.c_uint64, _P, _P, _P]),
    "kups_proposal_log_density": (_I32, [_P, _P, _I32, _P, _I64, _P, _P]),
    "kups_lj_tail_correction": (_I32, [_P, _P, _I32, _P, _P, _P, _P, _I32, _P, _P, _P, _P, _P]),
    "kups_gemm_bf16": (_I32, [_P, _I32, _I64, _I64, _P, _I32, _I64, _I64, _P, _I32, _I64, _I64, _P, _I32, _I64,
                               _I64, _P, _P, _I32, _I64, _I64, _I32, _I32, _I32, C.c_float, C.c_float, _I32, _I32, _P, _P]),
    "kups_bonded_order": (_I32, [_I32]),
    "kups_bonded_param_count": (_I32, [_I32]),
    "kups_bonded_edges": (_I32, [_I32, _P, _P, _P, _I64, _P, _I32, _P, _P, _I64, _P, _I32, _P, _P, _P, _I32, _P, _P]),
    "kups_bonded_delta_workspace_bytes": (_SZ, [_I64]),
    "kups_bonded_delta": (_I32, [_I32, _P, _P, _P, _I64, _P, _I32, _P, _P, _I64, _P, _I32, _P, _P, _P, _P, _P, _I64,
                                 _P, _I32, _P, _SZ, _P, _P]),
    "kups_erfc_eval": (_I32, [_P, _I64, _P, _P]),
    "kups_pair_edges": (_I32, [_P, _P, _P, _P, _I64, _P, _I32, _P, _P, _I32, _P, _P, _P, C.c_double, _I32, _P, _P, _I64, _P, _P, _P, _P, _P]),
}

_lib = None


class KupsError(RuntimeError):
    pass


class CapacityError(KupsError):
    """A device buffer was too small; ``required`` is the size that suffices."""

    def __init__(self, which: str, required: int, first_bad: int):
        super().__init__(f"capacity '{which}' exceeded: {required} required (first offender {first_bad})")
        self.which = which
        self.required = int(required)
        self.first_bad = int(first_bad)


def load(path: str | None = None):
    """Load (building first if needed) the shared library; raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build

        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != KUPS_OK:
        msg = load().kups_error_string(rc).decode()
        raise KupsError(f"{what}: {msg} (code {rc})")


def raise_status(st: Status) -> None:
    """Turn a device status word (already copied to the host) into an exception."""
    if st.code == KUPS_OK:
        return
    if st.code == KUPS_ERR_CAPACITY:
        raise CapacityError(CAPACITY_NAMES.get(st.detail, str(st.detail)), st.required, st.first_bad)
    msg = load().kups_error_string(st.code).decode()
    raise KupsError(f"device error: {msg} (code {st.code}, first offender {st.first_bad})")
