"""CPU checks of the C ABI library and the host logic (no GPU needed)."""

import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(kups_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    from kups_gb300 import _lib, build

    build.build()
    lib = _lib.load()
    declared = _declared_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    assert declared == set(_lib.SIGNATURES), "ctypes signature table out of sync with the header"
    assert lib.kups_version().startswith(b"kups_gb300")
    assert lib.kups_lj_md_max_atoms() == 2048


def test_error_strings():
    from kups_gb300 import _lib

    lib = _lib.load()
    for code in range(6):
        assert len(lib.kups_error_string(code)) > 0


def test_status_to_exception():
    from kups_gb300 import _lib

    _lib.raise_status(_lib.Status(0, 0, 0, -1))
    with pytest.raises(_lib.CapacityError) as e:
        _lib.raise_status(_lib.Status(_lib.KUPS_ERR_CAPACITY, _lib.KUPS_CAP_EDGES, 1234, 7))
    assert e.value.required == 1234 and e.value.which == "edges"


def test_workload_min_separation_and_shapes():
    from kups_gb300 import workloads
    from oracle import neighborlist as nl

    W = workloads.batched_uneven_lj(n_systems=24, seed=5)
    counts = np.bincount(W.system)
    assert counts.min() >= 64 and counts.max() <= 2048
    for s in range(24):
        m = W.system == s
        e, _ = nl.neighbor_list(W.positions[m], np.zeros(m.sum(), int), W.tril[s:s + 1], [0.9 * 3.405 - 1e-9])
        assert len(e) == 0


def test_key_to_seed_is_deterministic():
    from kups_gb300.md import key_to_seed

    assert key_to_seed([1, 2]) == key_to_seed([1, 2]) != key_to_seed([2, 1])


def test_struct_layouts_match_the_header(tmp_path):
    """Compile a C program against include/kups_gb300.h and compare sizeof / offsetof of every
    ABI struct with the ctypes mirrors (no GPU needed)."""
    import ctypes
    import os
    import shutil
    import subprocess

    from kups_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    structs = {"kups_status": _lib.Status, "kups_md_args": _lib.MdArgs, "kups_gcmc_proposal": _lib.GcmcProposal,
               "kups_gcmc_args": _lib.GcmcArgs, "kups_mlp": _lib.Mlp}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kups_gb300.h"', 'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_host_side_validation_of_newer_entry_points():
    """Arguments the library refuses before touching the device: an unknown bonded kind, an
    unknown MD integrator, a CSVR / NPT call without its thermostat or cell buffers, lanes per
    atom other than 1, 2 or 4, and undefined real-space term bits."""
    import ctypes as C

    from kups_gb300 import _lib

    lib = _lib.load()
    assert lib.kups_bonded_order(2) == 3 and lib.kups_bonded_param_count(4) == 3
    assert lib.kups_bonded_order(6) == -1
    assert lib.kups_bonded_edges(6, None, None, None, 0, None, 0, None, None, 1, None, 1, None, None, None, 0, None,
                                 None) == _lib.KUPS_ERR_INVALID
    assert lib.kups_bonded_edges(0, None, None, None, 0, None, 0, None, None, 0, None, 1, None, None, None, 1, None,
                                 None) == _lib.KUPS_OK  # no edges: nothing to do
    delta_args = lambda kind, n_changed, ws_bytes, ptr=None, inc=None: (
        [kind, ptr, ptr, ptr, 2, ptr, 1, ptr, ptr, 1, ptr, 1, inc, inc, ptr, ptr, None, n_changed, ptr, 0, ptr,
         ws_bytes, ptr, None])
    assert lib.kups_bonded_delta(*delta_args(6, 1, 0)) == _lib.KUPS_ERR_INVALID
    assert lib.kups_bonded_delta(*delta_args(0, 0, 0)) == _lib.KUPS_OK  # nothing moved
    assert lib.kups_bonded_delta(*delta_args(0, 1 << 31, 0)) == _lib.KUPS_ERR_INVALID  # beyond int32 slots
    # nothing below is dereferenced: each call is refused on the host
    assert lib.kups_bonded_delta(*delta_args(0, 1, 4, ptr=8)) == _lib.KUPS_ERR_INVALID  # workspace too small
    assert lib.kups_bonded_delta_workspace_bytes(10) >= 40
    a = _lib.MdArgs()
    a.n_systems, a.n_species, a.n_steps, a.neighbor_capacity = 1, 1, 1, 64
    for integrator, fields in ((4, {}), (2, {}), (3, {"thermostat_tau": 8})):
        a.integrator = integrator
        for k, v in fields.items():
            setattr(a, k, v)
        assert lib.kups_lj_md_run(C.byref(a), None, 0, None, None) == _lib.KUPS_ERR_INVALID
    assert lib.kups_lj_ewald_real_forces_packed(None, None, None, None, 1, 1, None, None, None, 1, None, None, None,
                                                1.0, 4, None, None, None, 0, None, None) == _lib.KUPS_ERR_INVALID
    assert lib.kups_lj_ewald_real_forces_packed(None, None, None, None, 1, 1, None, None, None, 1, None, None, None,
                                                1.0, 2 | 16, None, None, None, 0, None, None) == _lib.KUPS_ERR_INVALID


def test_host_side_validation_of_the_virial_observables():
    """kups_virial_stress refuses negative sizes, a kinetic energy without momenta, a
    molecular stress without groups and a short workspace; no systems is a no-op."""
    from kups_gb300 import _lib

    lib = _lib.load()
    ws = lib.kups_virial_stress_workspace_bytes(2, 3)
    assert ws >= 8 * 19 * 2 + 8 * 4 * 3 + 4 * 3 and lib.kups_virial_stress_workspace_bytes(-1, 0) == 0
    args = lambda **kw: [kw.get(k) for k in ("pos", "grad", "sys")] + [kw.get("n", 0), kw.get("tril"), None,
                                                                       kw.get("S", 0), kw.get("group"), kw.get("G", 0),
                                                                       kw.get("mom"), kw.get("mass"), None,
                                                                       kw.get("mol"), None, kw.get("kin"), None,
                                                                       kw.get("ws"), kw.get("wsb", 0), None, None]
    fake = 256  # never dereferenced: every call below is refused (or a no-op) on the host
    assert lib.kups_virial_stress(*args(n=-1)) == _lib.KUPS_ERR_INVALID
    assert lib.kups_virial_stress(*args(S=1)) == _lib.KUPS_ERR_INVALID  # no cell
    assert lib.kups_virial_stress(*args(S=1, tril=fake, kin=fake, wsb=1 << 20, ws=fake)) == _lib.KUPS_ERR_INVALID
    assert lib.kups_virial_stress(*args(S=1, tril=fake, mol=fake, wsb=1 << 20, ws=fake)) == _lib.KUPS_ERR_INVALID
    assert lib.kups_virial_stress(*args(S=1, tril=fake, wsb=16, ws=fake)) == _lib.KUPS_ERR_INVALID
    assert lib.kups_virial_stress(*args(n=4, pos=fake, grad=fake, sys=fake, S=1, tril=fake, wsb=1 << 20,
                                        ws=fake)) == _lib.KUPS_ERR_INVALID  # no status word
    assert lib.kups_virial_stress(*args()) == _lib.KUPS_OK
