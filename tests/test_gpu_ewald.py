"""GPU parity of the Ewald kernels against the float64 oracle.

Bars: the NaCl Madelung constant at the reference's rtol 5e-5
(test/potential/test_ewald.py:272-335); real-space pair terms in float64 within
rtol 1e-10; reciprocal space (float32 phase tables, float64 structure-factor
accumulation) within relative 1e-6 in energy and S(k), force RMS relative
error 1e-5, cell gradient relative 1e-5.
"""

import numpy as np
import pytest
import torch

from oracle import ewald as oew
from oracle import lennard_jones as olj
from oracle import neighborlist as onl
from oracle import unitcell as ouc
from oracle.units import TO_STANDARD_UNITS as KE

pytestmark = pytest.mark.gpu


def cuda(x, dtype=None):
    return torch.as_tensor(np.asarray(x), dtype=dtype).cuda()


def offsets(system, s):
    c = np.bincount(system, minlength=s)
    o = np.zeros(s + 1, np.int32)
    o[1:] = np.cumsum(c)
    return cuda(o, torch.int32), int(c.max())


def ionic_batch(seed=0):
    rng = np.random.default_rng(seed)
    pos, q, sysi, trils = [], [], [], []
    for s in range(2):
        L = ouc.lattice_from_lengths_angles(rng.uniform(12, 16, 3), rng.uniform(80, 100, 3))
        n = 40 + 10 * s
        f = rng.uniform(-0.5, 0.5, (n, 3))
        pos.append(f @ L)
        qq = rng.normal(0, 1, n)
        q.append(qq - qq.mean())
        sysi += [s] * n
        trils.append(ouc.tril_from_lattice(L))
    return np.concatenate(pos), np.concatenate(q), np.array(sysi), np.stack(trils)


def test_recip_matches_oracle():
    from kups_gb300.ewald import ewald_recip

    pos, q, sysi, tril = ionic_batch(1)
    kn = np.stack([oew.kvecs_cube(5)] * 2)
    alpha = np.array([0.3, 0.35])
    e, g, dt, sk = oew.long_range(pos, q, sysi, tril, kn, alpha)
    off, mx = offsets(sysi, 2)
    ge, gg, gdt, gsk, _ = ewald_recip(cuda(pos), cuda(q), off, mx, cuda(tril), cuda(kn, torch.int32), cuda(alpha))
    ge, gg, gdt, gsk = (x.cpu().numpy() for x in (ge, gg, gdt, gsk))
    np.testing.assert_allclose(ge, e, rtol=1e-6)
    np.testing.assert_allclose(gsk, sk, atol=2e-6 * np.abs(sk).max())
    rms = np.sqrt(np.mean((gg - g) ** 2) / np.mean(g**2))
    assert rms < 1e-5, rms
    np.testing.assert_allclose(gdt, dt, rtol=1e-5, atol=1e-5 * np.abs(dt).max())


def test_pair_edges_match_oracle():
    from kups_gb300.ewald import TERM_EWALD_REAL, TERM_LJ, TERM_VACUUM, pair_edges

    pos, q, sysi, tril = ionic_batch(2)
    rng = np.random.default_rng(3)
    sp = rng.integers(0, 2, len(q))
    sig, eps = olj.lorentz_berthelot([1.0, 1.3], [0.01, 0.02])
    rc = np.array([5.5, 6.0])
    e, s = onl.neighbor_list(pos, sysi, tril, rc)
    alpha = np.array([0.3, 0.35])
    el, gl, tl = olj.lj_from_edges(pos, sysi, sp, tril, sig, eps, rc, e, s)
    ee, ge, te = oew.short_range_from_edges(pos, q, sysi, tril, alpha, rc, e, s)
    en, gg, gt = pair_edges(cuda(pos), cuda(sysi), cuda(sp), cuda(q), cuda(tril), cuda(e, torch.int32),
                            cuda(s, torch.int32), len(e), TERM_LJ | TERM_EWALD_REAL, cuda(sig), cuda(eps), cuda(rc),
                            cuda(alpha), cuda(rc))
    np.testing.assert_allclose(en.cpu().numpy(), el + ee, rtol=1e-10)
    np.testing.assert_allclose(gg.cpu().numpy(), gl + ge, rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(gt.cpu().numpy(), tl + te, rtol=1e-9, atol=1e-10)
    # exclusion correction over explicit edges (ewald.py:328-346)
    xe = np.array([[0, 1], [1, 0], [2, 3], [3, 2]])
    xs = np.zeros((4, 3), np.int64)
    exp = oew.short_range_from_edges(pos, q, sysi, tril, alpha, [np.inf] * 2, xe, xs)[0] - \
        oew.coulomb_vacuum_from_edges(pos, q, sysi, tril, xe, xs, 2)
    got, _, _ = pair_edges(cuda(pos), cuda(sysi), None, cuda(q), cuda(tril), cuda(xe, torch.int32), cuda(xs, torch.int32),
                           4, TERM_EWALD_REAL | TERM_VACUUM, alpha=cuda(alpha), ewald_cutoff=cuda([np.inf, np.inf]))
    np.testing.assert_allclose(got.cpu().numpy(), exp, rtol=1e-10)


def test_madelung_on_gpu():
    from kups_gb300 import ewald

    cell = np.array([[0, 0, 0], [1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    tril, pos, q = ouc.make_supercell(ouc.tril_from_lattice(np.eye(3) * 2.0), 5, cell, np.array([-1.0] * 4 + [1.0] * 4))
    est = ewald.estimate_ewald_parameters(q, tril, epsilon_total=5e-5)
    prm = ewald.EwaldParameters(torch.tensor([est["alpha"]]), torch.tensor([est["real_cutoff"]]),
                                torch.as_tensor(ewald.kvecs_from_kmax(tril, est["k_max"]))[None])
    pot = ewald.LJEwaldPotential(prm)
    out = pot(ewald.EwaldParticles(cuda(pos), cuda(q), cuda(np.zeros(len(q), np.int32))), cuda(tril[None]))
    total = out.total_energies.cpu().numpy()[0] / KE
    assert np.isclose(-1.7475646 * 5**3 * 4, total, rtol=5e-5), total


def test_lj_ewald_potential_matches_oracle_sum():
    from kups_gb300 import ewald

    pos, q, sysi, tril = ionic_batch(4)
    sig, eps = olj.lorentz_berthelot([1.0, 1.2], [0.005, 0.01])
    sp = (np.arange(len(q)) % 2).astype(np.int32)
    kn = np.stack([oew.kvecs_cube(4)] * 2)
    alpha, rc = np.array([0.32, 0.32]), np.array([5.5, 5.5])
    prm = ewald.EwaldParameters(torch.tensor(alpha), torch.tensor(rc), torch.as_tensor(kn, dtype=torch.int32))
    pot = ewald.LJEwaldPotential(prm, sig, eps, rc)
    out = pot(ewald.EwaldParticles(cuda(pos), cuda(q), cuda(sysi, torch.int32), cuda(sp, torch.int32)), cuda(tril))
    e, s = onl.neighbor_list(pos, sysi, tril, rc)
    tot = olj.lj_from_edges(pos, sysi, sp, tril, sig, eps, rc, e, s)[0] + \
        oew.short_range_from_edges(pos, q, sysi, tril, alpha, rc, e, s)[0] + \
        oew.long_range(pos, q, sysi, tril, kn, alpha)[0] + oew.self_energy(q, sysi, alpha, 2)
    np.testing.assert_allclose(out.total_energies.cpu().numpy(), tot, rtol=1e-6)


def test_lj_ewald_md_conserves_energy_with_graph_replay():
    from kups_gb300 import ewald
    from kups_gb300.units import FEMTO_SECOND, KILO_CALORIE, MOL
    from kups_gb300.workloads import lattice_positions

    rng = np.random.default_rng(5)
    n, box = 216, 20.0
    pos = lattice_positions(rng, n, box, 2.2)
    q = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    sp = (np.arange(n) % 2).astype(np.int32)
    kcal = KILO_CALORIE / MOL
    sig, eps = olj.lorentz_berthelot([2.35, 4.40], [0.1 * kcal, 0.15 * kcal])
    masses = np.where(sp == 0, 22.99, 35.45)
    mom = rng.normal(0, 1, (n, 3)) * np.sqrt(masses * 300 * 8.617e-5)[:, None]
    tril = np.array([[box, 0, box, 0, 0, box]])
    prm = ewald.EwaldParameters(torch.tensor([0.3]), torch.tensor([9.0]), torch.as_tensor(oew.kvecs_cube(6)[None], dtype=torch.int32))
    parts = ewald.EwaldParticles(cuda(pos), cuda(q), cuda(np.zeros(n, np.int32)), cuda(sp))
    md = ewald.LJEwaldMD(parts, cuda(masses), cuda(tril), prm, 0.5 * FEMTO_SECOND, sig, eps, [9.0])
    md.start(cuda(mom))
    e0 = float((md.energy + md.kinetic_energy()).item())
    md.run(200)
    torch.cuda.synchronize()
    md.check()
    e1 = float((md.energy + md.kinetic_energy()).item())
    assert abs(e1 - e0) / abs(e0) < 2e-3, (e0, e1)


@pytest.mark.parametrize("binned", [False, True])
def test_allpairs_real_space_matches_edge_sum(binned):
    """kups_lj_ewald_real_forces (all pairs) and kups_lj_ewald_real_forces_packed (Morton-
    sorted atoms, partner groups skipped by box distance), float32 pair arithmetic, against
    the float64 oracle sum over the neighbour list at the cutoff: energy relative 1e-5,
    force RMS relative 1e-5; a cell narrower than twice the cutoff is refused
    (KUPS_ERR_UNSUPPORTED)."""
    import ctypes as C

    from kups_gb300 import _lib
    from kups_gb300.ewald import TERM_EWALD_REAL, TERM_LJ
    from kups_gb300.neighborlist import new_status, read_status

    rng = np.random.default_rng(9)
    pos, q, sysi, trils = [], [], [], []
    for s, n in enumerate((150, 230)):
        L = ouc.lattice_from_lengths_angles(rng.uniform(17, 20, 3), rng.uniform(85, 95, 3))
        from kups_gb300.workloads import lattice_positions

        f = lattice_positions(rng, n, 1.0, 0.1)  # fractional, min separation 0.1 of the cell
        pos.append((f - 0.5) @ L)
        qq = rng.normal(0, 1, n)
        q.append(qq - qq.mean())
        sysi += [s] * n
        trils.append(ouc.tril_from_lattice(L))
    pos, q, sysi, tril = np.concatenate(pos), np.concatenate(q), np.array(sysi), np.stack(trils)
    sp = rng.integers(0, 2, len(q)).astype(np.int32)
    sig, eps = olj.lorentz_berthelot([1.6, 2.0], [0.004, 0.006])
    rc = np.array([7.5, 8.0])
    alpha = np.array([0.35, 0.33])
    e, s = onl.neighbor_list(pos, sysi, tril, rc)
    el, gl, _ = olj.lj_from_edges(pos, sysi, sp, tril, sig, eps, rc, e, s)
    ee, ge, _ = oew.short_range_from_edges(pos, q, sysi, tril, alpha, rc, e, s)
    off, mx = offsets(sysi, 2)
    en = torch.empty(2, dtype=torch.float64, device="cuda")
    gr = torch.empty((len(q), 3), dtype=torch.float64, device="cuda")
    st = new_status()
    args = [cuda(pos), cuda(q), cuda(sp, torch.int32), off, cuda(tril), cuda(sig), cuda(eps), cuda(rc), cuda(alpha)]
    lib = _lib.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws = torch.empty(lib.kups_lj_ewald_real_forces_workspace_bytes(2, mx), dtype=torch.uint8, device="cuda")

    def real(rcut, status):
        common = (args[0].data_ptr(), args[1].data_ptr(), args[2].data_ptr(), off.data_ptr(), 2, mx,
                  args[4].data_ptr(), args[5].data_ptr(), args[6].data_ptr(), 2, rcut.data_ptr(), args[8].data_ptr(),
                  rcut.data_ptr(), KE, TERM_LJ | TERM_EWALD_REAL, en.data_ptr(), gr.data_ptr())
        if binned:
            return lib.kups_lj_ewald_real_forces_packed(*common, ws.data_ptr(), ws.numel(), status.data_ptr(), stream)
        return lib.kups_lj_ewald_real_forces(*common, status.data_ptr(), stream)

    rc_ = real(args[7], st)
    assert rc_ == 0
    torch.cuda.synchronize()
    assert read_status(st).code == 0
    np.testing.assert_allclose(en.cpu().numpy(), el + ee, rtol=1e-5)
    g = gl + ge
    rms = np.sqrt(np.mean((gr.cpu().numpy() - g) ** 2) / np.mean(g**2))
    assert rms < 1e-5, rms
    if binned:  # terms & 8: added onto the caller's energy and gradient
        e1, g1 = en.clone(), gr.clone()
        en.fill_(1.0)
        gr.fill_(1.0)
        lib.kups_lj_ewald_real_forces_packed(
            args[0].data_ptr(), args[1].data_ptr(), args[2].data_ptr(), off.data_ptr(), 2, mx, args[4].data_ptr(),
            args[5].data_ptr(), args[6].data_ptr(), 2, args[7].data_ptr(), args[8].data_ptr(), args[7].data_ptr(),
            KE, TERM_LJ | TERM_EWALD_REAL | 8, en.data_ptr(), gr.data_ptr(), ws.data_ptr(), ws.numel(),
            st.data_ptr(), stream)
        torch.cuda.synchronize()
        torch.testing.assert_close(en - 1.0, e1, rtol=1e-12, atol=1e-9)
        torch.testing.assert_close(gr - 1.0, g1, rtol=1e-6, atol=1e-9)
    # cutoff above half the narrowest width: refused, status records it
    st2 = new_status()
    big = cuda(np.array([9.9, 10.0]))
    real(big, st2)
    torch.cuda.synchronize()
    assert read_status(st2).code == _lib.KUPS_ERR_UNSUPPORTED


def test_pair_term_erfc_accuracy():
    """The library's erfc (Numerical Recipes' Chebyshev fit, float32) against float64 erfc on
    [0, 6]: relative error below 2e-6 for x <= 4 (alpha r reaches about 3.6 at the cutoffs used
    here) and below (x^2 + 2) 2^-23 + 1e-6 beyond, the exponential's argument rounding."""
    import ctypes as C

    from kups_gb300 import _lib

    x = torch.linspace(0.0, 6.0, 200001, dtype=torch.float32, device="cuda")
    out = torch.empty_like(x)
    assert _lib.load().kups_erfc_eval(x.data_ptr(), x.numel(), out.data_ptr(),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    ref = torch.special.erfc(x.double())
    rel = (out.double() - ref).abs() / ref
    xs = x.double()
    bound = torch.where(xs <= 4.0, torch.full_like(xs, 2e-6), (xs * xs + 2.0) * 2.0**-23 + 1e-6)
    keep = ref > 1e-15
    assert bool((rel[keep] < bound[keep]).all()), float((rel / bound)[keep].max())


def test_lj_ewald_md_baoab_graph_replays_the_eager_steps():
    """The captured BAOAB step of LJEwaldMD reads its Langevin counter from the device, so graph
    replays continue the eager trajectory's noise sequence (with a frozen counter the replayed
    steps would repeat one noise draw and leave it at once)."""
    from kups_gb300 import ewald
    from kups_gb300.autotune import autotune_lj_ewald
    from kups_gb300.units import FEMTO_SECOND

    rng = np.random.default_rng(5)
    n = 400
    L = ouc.lattice_from_lengths_angles([26.0, 27.0, 25.0], [90, 90, 90])
    g = np.stack(np.meshgrid(*[np.arange(8)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = (g + 0.5 + rng.uniform(-0.1, 0.1, g.shape)) / 8.0 @ L
    q = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    sp = (np.arange(n) % 2).astype(np.int32)
    masses = np.where(sp == 0, 22.99, 35.45)
    kn = oew.kvecs_cube(4)[None].astype(np.int32)
    prm = ewald.EwaldParameters(torch.tensor([0.3]), torch.tensor([9.0]), torch.as_tensor(kn))
    sig = np.array([[2.35, 2.6], [2.6, 2.9]])  # below the 3.2 A lattice spacing: a gentle start
    eps = np.array([[0.0043, 0.0053], [0.0053, 0.0065]])

    def make():
        parts = ewald.EwaldParticles(cuda(pos), cuda(q), cuda(np.zeros(n), torch.int32), cuda(sp, torch.int32))
        sim = ewald.LJEwaldMD(parts, cuda(masses), cuda(ouc.tril_from_lattice(L)[None]), prm, 1.0 * FEMTO_SECOND,
                              sig, eps, [9.0], integrator="baoab", temperature=1000.0, friction=0.01 / FEMTO_SECOND,
                              seed=3)
        sim.start(torch.zeros((n, 3), dtype=torch.float64, device="cuda"))
        return sim

    eager, graph = make(), make()
    assert eager.allpairs
    autotune_lj_ewald(graph, calls=3)
    eager.real_splits = graph.real_splits
    eager.run(6, use_graph=False)
    graph.run(6)
    torch.cuda.synchronize()
    assert int(graph.counter.item()) == 6 and int(eager.counter.item()) == 6
    np.testing.assert_allclose(graph.mom.cpu().numpy(), eager.mom.cpu().numpy(), rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(graph.p.positions.cpu().numpy(), eager.p.positions.cpu().numpy(), atol=1e-8)
