"""kups_ewald_recip_static (fixed scratch array, no workspace) against kups_ewald_recip.

Both entry points run the same kernels; only the order of the float64 atomic
additions into S(k) can differ, so the bar is relative 1e-12.  Two static
calls in a row with different sizes check that the second call does not
depend on what the first left in the shared array.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _batch(seed, n_systems, kmax, n_kvecs=None, empty=False):
    from oracle import ewald as oew
    from oracle import unitcell as ouc

    rng = np.random.default_rng(seed)
    pos, q, counts, trils = [], [], [], []
    for s in range(n_systems):
        L = ouc.lattice_from_lengths_angles(rng.uniform(11, 15, 3), rng.uniform(80, 100, 3))
        n = 0 if empty else int(rng.integers(20, 70))
        pos.append(rng.uniform(-0.5, 0.5, (n, 3)) @ L)
        qq = rng.normal(0, 1, n)
        q.append(qq - qq.mean())
        counts.append(n)
        trils.append(ouc.tril_from_lattice(L))
    off = np.zeros(n_systems + 1, np.int32)
    off[1:] = np.cumsum(counts)
    kv = oew.kvecs_cube(kmax)[: n_kvecs]
    kn = np.stack([kv] * n_systems).astype(np.int32).reshape(n_systems, len(kv), 3)
    alpha = rng.uniform(0.28, 0.36, n_systems)
    dev = lambda x, dt: torch.as_tensor(np.ascontiguousarray(x), dtype=dt).cuda()
    return dict(pos=dev(np.concatenate(pos).reshape(-1, 3), torch.float64), q=dev(np.concatenate(q), torch.float64),
                off=dev(off, torch.int32), max_atoms=max(counts), tril=dev(np.stack(trils), torch.float64),
                kn=dev(kn, torch.int32), alpha=dev(alpha, torch.float64))


def _outputs(b):
    s, nk = b["tril"].shape[0], b["kn"].shape[1]
    n = b["pos"].shape[0]
    f = lambda *shape: torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
    return f(s), f(n, 3), f(s, 6), f(s, nk, 2)


def _call(lib, b, static):
    from kups_gb300.neighborlist import new_status, read_status
    from kups_gb300.units import TO_STANDARD_UNITS

    e, g, gt, sk = _outputs(b)
    st = new_status()
    s, nk = b["tril"].shape[0], b["kn"].shape[1]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    head = (b["pos"].data_ptr(), b["q"].data_ptr(), b["off"].data_ptr(), s, b["max_atoms"], b["tril"].data_ptr(),
            b["kn"].data_ptr(), nk, b["alpha"].data_ptr(), TO_STANDARD_UNITS, e.data_ptr(), g.data_ptr(),
            gt.data_ptr(), sk.data_ptr())
    if static:
        rc = lib.kups_ewald_recip_static(*head, st.data_ptr(), stream)
    else:
        nbytes = lib.kups_ewald_recip_workspace_bytes(s, nk)
        ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        rc = lib.kups_ewald_recip(*head, ws.data_ptr(), nbytes, st.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert read_status(st).code == 0
    return [x.cpu().numpy() for x in (e, g, gt, sk)]


def _close(a, b):
    for x, y in zip(a, b):
        assert np.isfinite(x).all()
        np.testing.assert_allclose(x, y, rtol=RTOL, atol=RTOL * (np.abs(y).max() if y.size else 0.0))


def test_static_scratch_matches_workspace_entry_point_twice():
    from kups_gb300 import _lib

    lib = _lib.load()
    big = _batch(11, 24, 6)  # 24 systems x 1183 k vectors: 0.9 MiB of scratch
    small = _batch(12, 5, 4)  # different sizes on the second call
    ref_big, ref_small = _call(lib, big, False), _call(lib, small, False)
    _close(_call(lib, big, True), ref_big)
    _close(_call(lib, small, True), ref_small)


def test_static_scratch_refuses_sizes_beyond_the_array():
    from kups_gb300 import _lib

    lib = _lib.load()
    assert lib.kups_ewald_recip_static(None, None, None, 600, 10, None, None, 1000, None, 1.0, None, None, None, None,
                                       None, None) == 1  # KUPS_ERR_CAPACITY, nothing launched


def _scratch_bytes(n_systems, n_kvecs):
    """Bytes of the fixed array a call needs: 120 B of cell data per system and 32 B per
    (system, k vector), each part rounded up to 256 bytes."""
    up = lambda x: (x + 255) // 256 * 256
    return up(120 * n_systems) + up(32 * n_systems * n_kvecs)


def test_static_scratch_at_and_just_past_its_size():
    """256 systems x 2044 k vectors fill all but 2 KiB of the 16 MiB array and run; one more k
    vector per system needs more than the array and is refused before any launch."""
    from kups_gb300 import _lib

    lib = _lib.load()
    limit = 16 << 20
    assert _scratch_bytes(256, 2044) <= limit < _scratch_bytes(256, 2045)
    fits = _batch(21, 256, 8, n_kvecs=2044)
    _close(_call(lib, fits, True), _call(lib, fits, False))
    past = _batch(22, 256, 8, n_kvecs=2045)
    from kups_gb300.units import TO_STANDARD_UNITS

    e, g, gt, sk = _outputs(past)
    rc = lib.kups_ewald_recip_static(past["pos"].data_ptr(), past["q"].data_ptr(), past["off"].data_ptr(), 256,
                                     past["max_atoms"], past["tril"].data_ptr(), past["kn"].data_ptr(), 2045,
                                     past["alpha"].data_ptr(), TO_STANDARD_UNITS, e.data_ptr(), g.data_ptr(),
                                     gt.data_ptr(), sk.data_ptr(), None, None)
    assert rc == _lib.KUPS_ERR_CAPACITY
    torch.cuda.synchronize()
    assert torch.isnan(e).all()  # nothing was launched


def test_static_scratch_without_k_vectors_or_atoms():
    """n_kvecs = 0 (no structure-factor or force kernels over k) and systems without atoms
    (no per-atom kernels) give what the workspace entry point gives."""
    from kups_gb300 import _lib

    lib = _lib.load()
    no_k = _batch(31, 6, 3, n_kvecs=0)
    _close(_call(lib, no_k, True), _call(lib, no_k, False))
    no_atoms = _batch(32, 4, 3, empty=True)
    _close(_call(lib, no_atoms, True), _call(lib, no_atoms, False))
