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
