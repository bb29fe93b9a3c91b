"""GPU parity of the neighbour list, LJ and fused-MD kernels against the CPU oracle.

Bars: neighbour-list edge sets bit-exact as sorted (i, j, shift) rows;
float64 pair arithmetic within rtol 1e-10 of the oracle; float32 pair
arithmetic within force RMS relative error 1e-5 and energy relative error
1e-5 of the float64 oracle evaluated at the same (float32-representable)
positions.
"""

from dataclasses import replace

import numpy as np
import pytest
import torch

from oracle import lennard_jones as olj
from oracle import md as omd
from oracle import neighborlist as onl
from oracle import unitcell as ouc

pytestmark = pytest.mark.gpu

FORCE_RMS_TOL = 1e-5
ENERGY_REL_TOL = 1e-5


def cuda(x, dtype=None):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


def gpu_edges(pos, system, tril, cutoffs, inclusion=None, exclusion=None, n_inclusion=None, avg_edges=64):
    from kups_gb300.neighborlist import CellListNeighborList, NeighborListPoints

    pts = NeighborListPoints(cuda(pos, torch.float64), cuda(system, torch.int32),
                             None if inclusion is None else cuda(inclusion, torch.int32),
                             None if exclusion is None else cuda(exclusion, torch.int32), n_inclusion)
    edges, _ = CellListNeighborList(avg_edges).call_and_fix(pts, None, cuda(tril, torch.float64),
                                                             cuda(cutoffs, torch.float64))
    idx, sh = edges.valid()
    return onl.sort_edges(idx.cpu().numpy(), sh.cpu().numpy()), edges


def assert_same_edges(got, exp):
    ge, gs = got
    ee, es = exp
    assert ge.shape == ee.shape, (ge.shape, ee.shape)
    np.testing.assert_array_equal(ge, ee)
    np.testing.assert_array_equal(gs, es)


def _cube(L, n=1):
    return np.repeat(ouc.tril_from_lattice(np.eye(3) * L)[None], n, axis=0)


# ------------------------------------------------------------------ neighbour list
GOLDEN_NL = [
    # (positions, system, lattice-or-tril, cutoffs, exclusion) from test/core/test_neighborlist.py
    (np.array([[0.0, 0, 0], [0.4, 0, 0]]), [0, 0], ouc.tril_from_lattice(np.diag([1.0, 10, 10]))[None], [0.8], None),
    (np.array([[0.0, 0, 0], [0.3, 0.3, 0.3]]), [0, 0], _cube(1.0), [0.8], None),
    (np.random.default_rng(42).uniform(0, 1, (5, 3)), [0] * 5, _cube(1.5), [1.2], None),
    (np.array([[0.0, 0, 0], [0.4, 0, 0], [0.0, 0, 0], [1.0, 0, 0]]), [0, 0, 1, 1],
     ouc.tril_from_lattice(np.stack([np.diag([1.0, 10.0, 10.0]), np.eye(3) * 10])), [0.8, 1.5], None),
    (np.array([[0.0, 0, 0], [0.3, 0.2, 0.1]]), [0, 0],
     ouc.tril_from_lattice(np.array([[1.0, 0, 0], [0.5, 0.866, 0], [0, 0, 10.0]]))[None], [0.8], None),
    (np.zeros((1, 3)), [0], _cube(0.5), [0.55], None),
    (np.array([[0.0, 0, 0], [0.3, 0, 0]]), [0, 0], _cube(1.0), [np.inf], None),
    (np.array([[0.1, 0.1, 0.1], [0.4, 0.1, 0.1]]), [0, 0], _cube(0.5), [0.4], [0, 0]),
    (np.random.default_rng(0).uniform(0, 10, (15, 3)), [0] * 15, _cube(10.0), [3.0], None),
]


@pytest.mark.parametrize("case", range(len(GOLDEN_NL)))
def test_nl_golden_cases_bit_exact(case):
    pos, sysi, tril, cut, excl = GOLDEN_NL[case]
    exp = onl.neighbor_list(pos, sysi, tril, cut, exclusion=excl)
    got, _ = gpu_edges(pos, sysi, tril, cut, exclusion=excl)
    assert_same_edges(got, exp)


def random_triclinic_batch(seed=0, n_sys=8):
    rng = np.random.default_rng(seed)
    pos, sysi, trils, cuts, excl, incl = [], [], [], [], [], []
    off = 0
    for s in range(n_sys):
        lengths = rng.uniform(6, 16, 3)
        angles = rng.uniform(70, 110, 3)
        L = ouc.lattice_from_lengths_angles(lengths, angles)
        t = ouc.tril_from_lattice(L)
        n = int(rng.integers(3, 60)) * 3
        f = rng.uniform(-0.7, 0.7, (n, 3))  # some outside the primary cell on purpose
        pos.append(f @ L)
        sysi += [s] * n
        trils.append(t)
        cuts.append(rng.uniform(2.0, 9.0))  # some need periodic images
        excl += list(off + np.arange(n) // 3)  # molecules of three
        inc = np.full(n, s)
        inc[rng.uniform(size=n) < 0.05] = n_sys  # a few invalid inclusion labels
        incl += list(inc)
        off += n
    return np.concatenate(pos), np.array(sysi), np.stack(trils), np.array(cuts), np.array(excl), np.array(incl)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_nl_random_triclinic_batches_bit_exact(seed):
    pos, sysi, tril, cut, excl, incl = random_triclinic_batch(seed)
    exp = onl.neighbor_list(pos, sysi, tril, cut, inclusion=incl, exclusion=excl, n_inclusion=len(tril))
    got, _ = gpu_edges(pos, sysi, tril, cut, inclusion=incl, exclusion=excl, n_inclusion=len(tril))
    assert_same_edges(got, exp)


def test_nl_batched_uneven_subset_bit_exact():
    from kups_gb300 import workloads

    W = workloads.batched_uneven_lj(n_systems=24, n_max=600, seed=3)
    cut = np.full(W.n_systems, W.cutoff)
    exp = onl.neighbor_list(W.positions, W.system, W.tril, cut)
    got, _ = gpu_edges(W.positions, W.system, W.tril, cut)
    assert_same_edges(got, exp)


def test_nl_capacity_overflow_reports_required_and_pads():
    from kups_gb300 import _lib
    from kups_gb300.neighborlist import CellListNeighborList, NeighborListPoints

    pos, sysi, tril, cut, excl, incl = random_triclinic_batch(5, 3)
    exp = onl.neighbor_list(pos, sysi, tril, cut, exclusion=excl)
    pts = NeighborListPoints(cuda(pos, torch.float64), cuda(sysi, torch.int32), None, cuda(excl, torch.int32))
    with pytest.raises(_lib.CapacityError) as err:
        CellListNeighborList(avg_edges=1)(pts, None, cuda(tril, torch.float64), cuda(cut, torch.float64))
    assert err.value.required == len(exp[0])
    got, edges = gpu_edges(pos, sysi, tril, cut, exclusion=excl, avg_edges=1)
    assert_same_edges(got, exp)
    tail = edges.indices[edges.n_edges:]
    assert bool((tail == len(pos)).all()) and bool((edges.shifts[edges.n_edges:] == 0).all())


# ------------------------------------------------------------------ LJ over edges
SIG = np.array([[1.0, 1.2], [1.2, 1.0]])
EPS = np.array([[1.0, 0.8], [0.8, 1.0]])


def test_lj_golden_pairs_on_gpu():
    from kups_gb300.potential import lj_from_edges

    cases = [
        (np.array([[0.0, 0, 0], [1.0, 0, 0]]), [0, 1], [[0, 1]], 4 * 0.8 * (1.2**12 - 1.2**6)),
        (np.array([[0.0, 0, 0], [1.5, 0, 0]]), [0, 0], [[0, 1]], 4 * ((1 / 1.5) ** 12 - (1 / 1.5) ** 6)),
    ]
    for pos, sp, e, expected in cases:
        for fp32 in (False, True):
            out = lj_from_edges(cuda(pos), cuda([0, 0]), cuda(sp), cuda(_cube(10.0)), cuda(SIG), cuda(EPS), cuda([12.0]),
                                cuda(e, torch.int32), cuda(np.zeros((1, 3)), torch.int32), 1, fp32)
            assert np.isclose(out.total_energies.cpu().numpy()[0] * 2, expected, rtol=1e-6)


@pytest.mark.parametrize("fp32", [False, True])
def test_lj_edges_match_oracle(fp32):
    from kups_gb300.potential import lj_from_edges

    rng = np.random.default_rng(7)
    pos, sysi, tril, cut, excl, incl = random_triclinic_batch(7, 4)
    # spread atoms so LJ stays moderate: sigma small relative to spacing
    sp = rng.integers(0, 2, len(pos))
    sig = SIG * 1.1
    e, s = onl.neighbor_list(pos, sysi, tril, cut)
    en, g, dt = olj.lj_from_edges(pos, sysi, sp, tril, sig, EPS, cut, e, s)
    out = lj_from_edges(cuda(pos), cuda(sysi), cuda(sp), cuda(tril), cuda(sig), cuda(EPS), cuda(cut), cuda(e, torch.int32),
                        cuda(s, torch.int32), len(e), fp32)
    ge = out.total_energies.cpu().numpy()
    gg = out.gradients.positions.cpu().numpy()
    gt = out.gradients.unitcell.cpu().numpy()
    if not fp32:
        np.testing.assert_allclose(ge, en, rtol=1e-10)
        np.testing.assert_allclose(gg, g, rtol=1e-9, atol=1e-9 * np.abs(g).max())
        np.testing.assert_allclose(gt, dt, rtol=1e-9, atol=1e-9 * np.abs(dt).max())
    else:
        assert np.all(np.abs(ge - en) <= ENERGY_REL_TOL * np.abs(en) + 1e-12)
        rms = np.sqrt(np.mean((gg - g) ** 2)) / np.sqrt(np.mean(g**2))
        assert rms <= FORCE_RMS_TOL, rms
        np.testing.assert_allclose(gt, dt, rtol=1e-4, atol=1e-5 * np.abs(dt).max())


# ------------------------------------------------------------------ fused MD
def md_state(W, forces=None):
    from kups_gb300 import md, potential

    prm = potential.LennardJonesParameters("Ar", torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(cuda(W.positions, torch.float64), cuda(W.momenta, torch.float64), cuda(W.masses, torch.float64),
                           cuda(W.species, torch.int32), cuda(W.system, torch.int32), forces)
    systems = md.MDSystems(cuda(W.tril, torch.float64), cuda(W.time_step), cuda(W.temperature), cuda(W.friction))
    return md.MDState(parts, systems, prm, skin=W.skin)


def small_batch():
    from kups_gb300 import workloads

    return workloads.batched_uneven_lj(n_systems=12, n_min=64, n_max=700, seed=11)


def oracle_forces(W, pos):
    cut = np.full(W.n_systems, W.cutoff)
    return omd.lj_forces(pos, W.system, W.species, W.tril, W.sigma, W.epsilon, cut)


@pytest.mark.parametrize("which", ["batch", "argon"])
def test_fused_md_forces_energy_virial_match_oracle(which):
    from kups_gb300 import md, workloads

    W = small_batch() if which == "batch" else workloads.argon_fcc()
    W.positions = W.positions + np.random.default_rng(1).normal(0, 0.1, W.positions.shape)
    state = md_state(W)
    prop = md.make_velocity_verlet_step(steps_per_call=0)
    out = prop(None, state)
    pos = out.particles.positions.cpu().numpy()
    e, f, dt = oracle_forces(W, pos)
    gf = out.particles.forces.cpu().numpy()
    ge = out.systems.potential_energy.cpu().numpy()
    gv = out.systems.unitcell_gradients.cpu().numpy()
    rms = np.sqrt(np.mean((gf - f) ** 2)) / np.sqrt(np.mean(f**2))
    assert rms <= FORCE_RMS_TOL, rms
    assert np.all(np.abs(ge - e) <= ENERGY_REL_TOL * np.abs(e)), (ge, e)
    np.testing.assert_allclose(gv, dt, rtol=1e-4, atol=1e-4 * np.abs(dt).max())


def test_fused_md_velocity_verlet_tracks_oracle():
    from kups_gb300 import md

    W = small_batch()
    state = md_state(W)
    prop = md.make_velocity_verlet_step(steps_per_call=10)
    # start both from the same float32-rounded state with forces at t = 0
    s0 = md.make_velocity_verlet_step(steps_per_call=0)(None, state)
    pos0 = s0.particles.positions.cpu().numpy()
    mom0 = s0.particles.momenta.cpu().numpy()
    _, f0, _ = oracle_forces(W, pos0)
    out = prop(None, s0)
    cut = np.full(W.n_systems, W.cutoff)
    pos, mom, _, _ = omd.velocity_verlet(pos0, mom0, f0, W.masses, W.system, W.species, W.tril, W.sigma, W.epsilon, cut,
                                         W.time_step, 10)
    gp = out.particles.positions.cpu().numpy()
    d = ouc.wrap(gp - pos, W.tril[W.system])
    assert np.abs(d).max() < 1e-3, np.abs(d).max()
    np.testing.assert_allclose(out.particles.momenta.cpu().numpy(), mom, atol=2e-3 * np.abs(mom).max())


def test_fused_md_is_deterministic():
    from kups_gb300 import md

    W = small_batch()
    outs = []
    for _ in range(2):
        prop = md.make_baoab_langevin_step(steps_per_call=25)
        o = prop([7, 9], md_state(W))
        outs.append((o.particles.positions.cpu().numpy(), o.systems.potential_energy.cpu().numpy()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_fused_md_capacity_retry_matches_large_capacity():
    from kups_gb300 import md

    W = small_batch()
    a = md.FusedLennardJonesMD("velocity_verlet", 5, neighbor_capacity=16)(None, md_state(W))
    b = md.FusedLennardJonesMD("velocity_verlet", 5, neighbor_capacity=256)(None, md_state(W))
    np.testing.assert_array_equal(a.particles.positions.cpu().numpy(), b.particles.positions.cpu().numpy())


def test_fused_md_baoab_thermostat_temperature():
    from kups_gb300 import md, workloads
    from kups_gb300.units import BOLTZMANN_CONSTANT

    W = workloads.batched_uneven_lj(n_systems=8, n_min=400, n_max=500, seed=4, friction_per_ps=20.0)
    prop = md.make_baoab_langevin_step()
    packed = md.pack(md_state(W))
    _, tke = prop.run_packed(packed, 1500, seed=3, trace=True)
    ke = tke.cpu().numpy()[500:].mean(axis=0)
    n = np.bincount(W.system)
    T = 2 * ke / (3 * n * BOLTZMANN_CONSTANT)
    np.testing.assert_allclose(T, W.temperature, rtol=0.06)


def test_lj_tail_correction_matches_oracle():
    """Global tail energy and pressure (lennard_jones.py:276-340) against the float64 oracle
    (relative 1e-12), with the default mask (eps > 0) and an explicit one."""
    import torch

    from kups_gb300.potential import lennard_jones_tail_correction
    from oracle import lennard_jones as olj
    from oracle import unitcell as ouc

    rng = np.random.default_rng(4)
    counts = [30, 55, 12]
    system = np.repeat(np.arange(3), counts).astype(np.int32)
    species = rng.integers(0, 3, len(system)).astype(np.int32)
    tril = np.stack([ouc.tril_from_lattice(ouc.lattice_from_lengths_angles(rng.uniform(15, 25, 3),
                                                                          rng.uniform(80, 100, 3))) for _ in range(3)])
    sig, eps = olj.lorentz_berthelot([3.0, 3.4, 2.6], [0.01, 0.0, 0.02])
    rc = np.array([10.0, 11.0, 12.0])
    sc = np.stack([np.bincount(species[system == s], minlength=3) for s in range(3)])
    for mask in (None, np.array([[1, 0, 1], [0, 1, 1], [1, 1, 0]])):
        e, p = lennard_jones_tail_correction(species, system, tril, sig, eps, rc, tail_mask=mask)
        m = None if mask is None else mask.astype(bool)
        np.testing.assert_allclose(e.cpu().numpy(), olj.tail_correction_energy(sc, tril, sig, eps, rc, m), rtol=1e-12)
        np.testing.assert_allclose(p.cpu().numpy(), olj.tail_correction_pressure(sc, tril, sig, eps, rc, m), rtol=1e-12)


def test_fused_md_pressure_matches_reference_formula():
    """Instantaneous pressure (md/observables.py:38-61) with the virial-theorem stress
    (observables/stress.py:70-82): P = 2K / 3V + Tr(sigma) / 3,
    sigma = -(sum_i dU/dr_i (x) r_i + h^T dU/dh) / V, from the float64 oracle's gradients at the
    returned positions (bar: relative 1e-4, float32 pair arithmetic)."""
    from kups_gb300 import md

    W = small_batch()
    out = md.make_baoab_langevin_step(steps_per_call=8)([3, 4], md_state(W))
    pos = out.particles.positions.cpu().numpy()
    mom = out.particles.momenta.cpu().numpy()
    e, f, dt = oracle_forces(W, pos)
    got = out.systems.pressure.cpu().numpy()
    exp = []
    for s in range(W.n_systems):
        sel = W.system == s
        L = ouc.lattice_from_tril(W.tril[s])
        G = np.zeros((3, 3))
        G[0, 0], G[1, 0], G[1, 1], G[2, 0], G[2, 1], G[2, 2] = dt[s]
        vol = abs(np.linalg.det(L))
        sigma = -((-f[sel])[:, :, None] * pos[sel][:, None, :]).sum(0)
        sigma -= L.T @ G
        sigma /= vol
        ke = 0.5 * np.sum(mom[sel] ** 2 / W.masses[sel][:, None])
        exp.append(2 * ke / (3 * vol) + np.trace(sigma) / 3)
    np.testing.assert_allclose(got, exp, rtol=1e-4, atol=1e-4 * np.abs(exp).max())


def _packed_copy(packed):
    from dataclasses import replace

    return replace(packed, pos4=packed.pos4.clone(), mom4=packed.mom4.clone(), frc4=packed.frc4.clone(),
                   energy=None, kinetic=None, virial=None, pressure=None,
                   rebuilds=torch.zeros(packed.n_systems, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("integrator", ["velocity_verlet", "baoab"])
def test_fused_md_resumes_lists_across_calls(integrator):
    """Two calls of 30 steps on one workspace give the state of one 60-step call bit for bit:
    the second call resumes every system from the workspace record (cell-sorted order, image
    copies, travelled distances, Verlet list) instead of rebuilding, so the list-build count
    of the split run equals the single run's."""
    from kups_gb300 import md

    W = small_batch()
    base = md.pack(md_state(W))
    one, two = _packed_copy(base), _packed_copy(base)
    md.FusedLennardJonesMD(integrator).run_packed(one, 60, seed=5, step0=0)
    prop = md.FusedLennardJonesMD(integrator)
    prop.run_packed(two, 30, seed=5, step0=0)
    first = two.rebuilds.clone()
    prop.run_packed(two, 30, seed=5, step0=30)
    for x, y in ((one.pos4, two.pos4), (one.mom4, two.mom4), (one.frc4, two.frc4)):
        np.testing.assert_array_equal(x.cpu().numpy(), y.cpu().numpy())
    np.testing.assert_array_equal(one.energy.cpu().numpy(), two.energy.cpu().numpy())
    np.testing.assert_array_equal(one.rebuilds.cpu().numpy(), two.rebuilds.cpu().numpy())
    assert int(first.min()) >= 1  # every system built its list in the first call


def test_fused_md_rebuilds_when_the_input_changed():
    """A system whose positions were changed between calls (or every system, with
    reuse_lists off) is rebuilt, and its forces still match the oracle."""
    from kups_gb300 import md

    W = small_batch()
    packed = _packed_copy(md.pack(md_state(W)))
    prop = md.make_velocity_verlet_step()
    prop.run_packed(packed, 10, seed=1, step0=0)
    off = packed.sys_offset.cpu().numpy()
    packed.pos4[off[3], 0] += 0.01  # move one atom of system 3
    packed.forces_valid = False
    packed.rebuilds.zero_()
    prop.run_packed(packed, 0, seed=1, step0=10)
    reb = packed.rebuilds.cpu().numpy()
    assert reb[3] == 1 and reb.sum() == 1, reb
    pos4 = packed.pos4.cpu().numpy()
    perm = packed.perm.cpu().numpy()
    pos = np.empty((len(perm), 3))
    pos[perm] = pos4[:, :3]
    e, f, _ = oracle_forces(W, pos)
    gf = np.empty((len(perm), 3))
    gf[perm] = packed.frc4.cpu().numpy()[:, :3]
    rms = np.sqrt(np.mean((gf - f) ** 2)) / np.sqrt(np.mean(f**2))
    assert rms <= FORCE_RMS_TOL, rms
    prop.reuse_lists = False
    packed.rebuilds.zero_()
    prop.run_packed(packed, 5, seed=1, step0=10)
    assert int(packed.rebuilds.cpu().numpy().min()) >= 1


def test_fused_md_per_step_virial_trace():
    """trace_virial holds dE/dtril after every step: its last row is the launch's virial bit for
    bit, and every row matches the float64 oracle at that step's positions (1e-4 relative)."""
    from kups_gb300 import md

    W = small_batch()
    prop = md.make_velocity_verlet_step()
    packed = md.pack(md_state(W))
    S = W.n_systems
    rows = []
    for k in range(3):
        tv = torch.zeros((2, S, 6), dtype=torch.float64, device="cuda")
        st = prop.launch(packed, 2, seed=1, step0=2 * k, trace_virial=tv)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(tv[-1].cpu().numpy(), packed.virial.cpu().numpy())
        pos = np.empty((packed.n_atoms, 3))
        pos[packed.perm.cpu().numpy()] = packed.pos4.cpu().numpy()[:, :3]
        _, _, dt = oracle_forces(W, pos)
        np.testing.assert_allclose(tv[-1].cpu().numpy(), dt, rtol=1e-4, atol=1e-4 * np.abs(dt).max())
        rows.append(tv[0].cpu().numpy())
    assert all(np.isfinite(r).all() for r in rows)


def test_pack_reuses_the_layout_of_unchanged_inputs():
    """md.pack(state, reuse=previous) takes the sort by system, offsets, queue order and
    per-system parameters from `previous` while the state's static objects are the same and
    unmodified, and packs the same arrays as a fresh pack; a modified input forces a fresh one."""
    from kups_gb300 import md, workloads

    W = workloads.batched_uneven_lj(n_systems=24, seed=3)
    state = md_state(W)
    first = md.pack(state)
    moved = replace(state, particles=replace(state.particles, positions=state.particles.positions + 0.01))
    again = md.pack(moved, reuse=first)
    fresh = md.pack(moved)
    assert again.perm is first.perm and again.order is first.order
    for f in ("pos4", "mom4", "perm", "sys_offset", "order", "tril32", "cutoff", "skin", "dt", "kT", "friction"):
        assert torch.equal(getattr(again, f), getattr(fresh, f)), f
    assert (again.max_atoms, again.max_density) == (fresh.max_atoms, fresh.max_density)
    state.particles.masses.mul_(1.0)  # an in-place write bumps the version: no reuse
    third = md.pack(moved, reuse=again)
    assert third.perm is not again.perm
