"""Degenerate inputs the reference's tests exercise, through the C ABI on the GPU.

* a single particle in a cell smaller than the cutoff sees its own periodic images and never
  itself (test/core/test_neighborlist.py:1040-1116);
* an infinite cutoff gives the minimum image only, no replication (:1118-1162);
* empty batches, empty systems between populated ones and a system of one atom;
* a cutoff needing more image offsets than the search allows is refused with
  KUPS_ERR_UNSUPPORTED and no edges, instead of running (the reference would materialise
  that many copies of every candidate pair);
* energies and forces of an empty edge set, and the fused MD on a batch holding a one-atom
  system, against the oracle.
"""

import math

import numpy as np
import pytest
import torch

from oracle import neighborlist as onl
from oracle import unitcell as ouc

pytestmark = pytest.mark.gpu


def cuda(x, dtype=None):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


def _nl(pos, system, tril, cutoffs, cap=64, exclusion=None):
    from kups_gb300 import _lib
    from kups_gb300.neighborlist import new_status, read_status

    lib = _lib.load()
    n, s = len(pos), len(tril)
    p = cuda(np.asarray(pos, np.float64).reshape(-1, 3), torch.float64)
    sysi = cuda(system, torch.int32)
    incl = torch.zeros(n, dtype=torch.int32, device="cuda") if n else torch.zeros(1, dtype=torch.int32, device="cuda")
    excl = cuda(np.arange(n) if exclusion is None else exclusion, torch.int32) if n else incl
    tr = cuda(np.asarray(tril, np.float64).reshape(-1, 6), torch.float64)
    cut = cuda(cutoffs, torch.float64)
    edges = torch.full((cap, 2), -7, dtype=torch.int32, device="cuda")
    shifts = torch.full((cap, 3), -7, dtype=torch.int32, device="cuda")
    ne = torch.zeros(1, dtype=torch.int64, device="cuda")
    ws = torch.empty(lib.kups_neighborlist_workspace_bytes(n, s), dtype=torch.uint8, device="cuda")
    st = new_status()
    rc = lib.kups_neighborlist_build(p.data_ptr(), sysi.data_ptr(), incl.data_ptr(), excl.data_ptr(), n, 1,
                                     tr.data_ptr(), cut.data_ptr(), s, edges.data_ptr(), shifts.data_ptr(), cap,
                                     ne.data_ptr(), ws.data_ptr(), ws.numel(), st.data_ptr(), None)
    _lib.check(rc, "kups_neighborlist_build")
    torch.cuda.synchronize()
    k = int(ne.item())
    return k, edges.cpu().numpy(), shifts.cpu().numpy(), read_status(st)


def _edge_set(k, e, sh):
    return {(int(a), int(b), tuple(int(x) for x in c)) for (a, b), c in zip(e[:k], sh[:k])}


def test_single_particle_sees_its_own_images():
    tril = ouc.tril_from_lattice(np.eye(3) * 0.5)[None]
    k, e, sh, st = _nl([[0.0, 0.0, 0.0]], [0], tril, [0.55])
    assert st.code == 0
    expected = {(0, 0, s) for s in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]}
    assert _edge_set(k, e, sh) == expected
    # the oracle's own rule agrees
    ref_e, ref_s = onl.neighbor_list(np.zeros((1, 3)), np.zeros(1, int), tril, np.array([0.55]))
    assert _edge_set(len(ref_e), np.asarray(ref_e), np.asarray(ref_s).reshape(-1, 3)) == expected


def test_infinite_cutoff_is_the_minimum_image_only():
    tril = ouc.tril_from_lattice(np.eye(3))[None]
    k, e, sh, st = _nl([[0.0, 0.0, 0.0], [0.3, 0.0, 0.0]], [0, 0], tril, [math.inf])
    assert st.code == 0
    assert _edge_set(k, e, sh) == {(0, 1, (0, 0, 0)), (1, 0, (0, 0, 0))}


def test_empty_batch_and_empty_systems():
    tril = np.stack([ouc.tril_from_lattice(np.eye(3) * 10.0)] * 4)
    # no particles at all: nothing found, every row padded with i = j = n = 0
    k, e, sh, st = _nl(np.zeros((0, 3)), np.zeros(0, int), tril, [3.0] * 4, cap=8)
    assert k == 0 and st.code == 0
    assert (e == 0).all() and (sh == 0).all()
    # systems 0 and 2 empty, system 1 one atom, system 3 two atoms 1 A apart
    pos = [[1.0, 1.0, 1.0], [2.0, 2.0, 2.0], [3.0, 2.0, 2.0]]
    k, e, sh, st = _nl(pos, [1, 3, 3], tril, [3.0] * 4, cap=8)
    assert st.code == 0
    assert _edge_set(k, e, sh) == {(1, 2, (0, 0, 0)), (2, 1, (0, 0, 0))}
    assert (e[k:] == 3).all() and (sh[k:] == 0).all()


def test_cutoff_of_many_cell_widths_is_refused():
    from kups_gb300 import _lib

    tril = np.stack([ouc.tril_from_lattice(np.eye(3) * 2.0), ouc.tril_from_lattice(np.eye(3) * 10.0)])
    pos = [[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [1.0, 1.0, 1.0], [2.0, 1.0, 1.0]]
    # system 0: a 2 A cell with a 50 A cutoff (51 images per axis); system 1 is ordinary
    k, e, sh, st = _nl(pos, [0, 0, 1, 1], tril, [50.0, 3.0], cap=16)
    assert st.code == _lib.KUPS_ERR_UNSUPPORTED and st.first_bad == 0
    assert _edge_set(k, e, sh) == {(2, 3, (0, 0, 0)), (3, 2, (0, 0, 0))}


def test_lj_of_no_edges_is_zero():
    from kups_gb300 import potential

    tril = ouc.tril_from_lattice(np.eye(3) * 30.0)[None]
    pos = np.array([[0.0, 0.0, 0.0], [10.0, 0.0, 0.0]])  # beyond the cutoff
    prm = potential.LennardJonesParameters(("A",), torch.tensor([[3.4]]), torch.tensor([[0.01]]),
                                           torch.tensor([5.0], dtype=torch.float64))
    st = potential.LJState(potential.LJParticles(cuda(pos, torch.float64), cuda([0, 0], torch.int32),
                                                 cuda([0, 0], torch.int32)), cuda(tril, torch.float64), prm)
    out = potential.LennardJonesPotential()(st)
    assert float(out.total_energies.abs().sum()) == 0.0
    assert float(out.gradients.positions.abs().sum()) == 0.0


def test_fused_md_with_a_one_atom_system_tracks_the_oracle():
    """A one-atom system (no pairs) drifts freely beside an ordinary one; both against the
    float64 oracle's velocity Verlet."""
    from kups_gb300 import md, potential, workloads
    from oracle import md as omd


    W = workloads.batched_uneven_lj(n_systems=2, n_min=64, n_max=100, seed=2)
    # replace system 0 by a single atom with a known momentum
    keep = W.system == 1
    pos = np.concatenate([[[1.0, 2.0, 3.0]], W.positions[keep]])
    mom = np.concatenate([[[0.3, -0.2, 0.1]], W.momenta[keep]])
    mass = np.concatenate([[39.948], W.masses[keep]])
    sysi = np.concatenate([[0], np.ones(keep.sum(), int)])
    spc = np.zeros(len(pos), np.int32)
    prm = potential.LennardJonesParameters("Ar", torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    state = md.MDState(md.MDParticles(cuda(pos, torch.float64), cuda(mom, torch.float64), cuda(mass, torch.float64),
                                      cuda(spc, torch.int32), cuda(sysi, torch.int32)),
                       md.MDSystems(cuda(W.tril, torch.float64), cuda(W.time_step), cuda(W.temperature),
                                    cuda(W.friction)), prm, skin=W.skin)
    # start both from the same float32-rounded state with forces at t = 0
    s0 = md.make_velocity_verlet_step(steps_per_call=0)(None, state)
    pos0, mom0 = s0.particles.positions.cpu().numpy(), s0.particles.momenta.cpu().numpy()
    cut = np.full(2, W.cutoff)
    _, f0, _ = omd.lj_forces(pos0, sysi, spc, W.tril, W.sigma, W.epsilon, cut)
    assert np.abs(f0[0]).max() == 0.0  # no partner
    out = md.make_velocity_verlet_step(steps_per_call=10)(None, s0)
    ref_pos, ref_mom, _, _ = omd.velocity_verlet(pos0, mom0, f0, mass, sysi, spc, W.tril, W.sigma, W.epsilon, cut,
                                                 W.time_step, 10)
    got = out.particles.positions.cpu().numpy()
    d = ouc.wrap(got - ref_pos, W.tril[sysi])
    assert np.abs(d).max() < 1e-3, np.abs(d).max()
    # the lone atom's momentum is untouched
    np.testing.assert_allclose(out.particles.momenta.cpu().numpy()[0], mom0[0], rtol=1e-6)
    np.testing.assert_allclose(out.particles.momenta.cpu().numpy(), ref_mom, atol=2e-3 * np.abs(ref_mom).max())
