"""GPU GCMC step: incremental energies against float64 full recomputation, and sampling checks.

Bars: each proposed move's energy change within 2e-5 eV + 2e-5 relative of
E_oracle(after) - E_oracle(before) (float32 pair arithmetic, float64 sums);
the ideal-gas limit (no interactions) reproduces the Poisson mean loading
<N> = a V within 4 standard errors.
"""

import numpy as np
import pytest
import torch

from oracle import gcmc as ogc
from oracle import unitcell as ouc

pytestmark = pytest.mark.gpu


def co2_template():
    return np.array([[0.0, 0, 0], [1.16, 0, 0], [-1.16, 0, 0]]), np.array([4, 5, 5]), np.array([0.70, -0.35, -0.35])


def small_setup(n_sys=2, seed=0, tail=True, charges=True, rc=7.0):
    from kups_gb300 import gcmc
    from kups_gb300.ewald import kvecs_from_kmax
    from kups_gb300.units import BOLTZMANN_CONSTANT

    rng = np.random.default_rng(seed)
    L = ouc.lattice_from_lengths_angles([12.0, 12.0, 13.0], [90, 90, 120])
    tril = ouc.tril_from_lattice(L)
    n_fw = 40
    fw_frac = rng.uniform(0, 1, (n_fw, 3))  # stored in [0, 1), as a CIF host would be
    fw_pos = fw_frac @ L
    fw_sp = rng.integers(0, 4, n_fw)
    q = rng.normal(0, 0.3, n_fw) if charges else np.zeros(n_fw)
    q -= q.mean()
    mpos, msp, mq = co2_template()
    if not charges:
        mq = np.zeros(3)
    sig_i = np.array([2.5, 2.9, 3.2, 3.5, 2.80, 3.05])
    eps_i = np.array([20, 40, 60, 80, 27, 79]) * BOLTZMANN_CONSTANT
    sigma, epsilon = gcmc.lorentz_berthelot(sig_i, eps_i)
    alpha = 0.35
    kn = kvecs_from_kmax(tril, 1.6)
    setup = gcmc.GCMCSetup(
        fw_positions=fw_pos, fw_species=fw_sp, fw_charges=q, fw_start=np.zeros(n_sys, int),
        fw_count=np.full(n_sys, n_fw), tril=np.repeat(tril[None], n_sys, 0), motif_positions=mpos,
        motif_species=msp, motif_charges=mq, sigma=sigma, epsilon=epsilon, rc_lj=np.full(n_sys, rc),
        rc_ew=np.full(n_sys, rc), alpha=np.full(n_sys, alpha), kvec_n=np.repeat(kn[None], n_sys, 0),
        temperature=np.full(n_sys, 298.0), log_activity=np.full(n_sys, -9.0), max_mol=16, tail_correction=tail)
    return setup


def oracle_energy(setup, guests):
    return ogc.total_energy(setup.fw_positions, setup.fw_species, setup.fw_charges, guests, setup.motif_species,
                            setup.motif_charges, setup.tril[0], setup.sigma, setup.epsilon, setup.rc_lj[0],
                            setup.rc_ew[0], setup.alpha[0], setup.kvec_n[0], tail=setup.tail_correction)


def random_molecule(rng, L, template):
    from scipy.spatial.transform import Rotation

    R = Rotation.random(random_state=rng.integers(1 << 30)).as_matrix()
    c = rng.uniform(-0.5, 0.5, 3) @ L
    return template @ R.T + c


def wrapped(p, tril):
    return ouc.wrap(p, tril)


@pytest.mark.parametrize("rc", [7.0, 5.0])  # 3 x 3 x 3 image offsets / minimum image (widths 10.4, 10.4, 13 A)
@pytest.mark.parametrize("kind", ["translate", "rotate", "reinsert", "insert", "delete"])
def test_move_energy_change_matches_oracle(kind, rc):
    from kups_gb300 import gcmc

    setup = small_setup(n_sys=3, rc=rc)
    rng = np.random.default_rng({"translate": 1, "rotate": 2, "insert": 3, "delete": 4, "reinsert": 5}[kind])
    L = ouc.lattice_from_tril(setup.tril[0])
    mpos = setup.motif_positions
    guests = [np.concatenate([wrapped(random_molecule(rng, L, mpos), setup.tril[0]) for _ in range(4)])
              for _ in range(3)]
    mc = gcmc.GCMC(setup, seed=5)
    mc.set_guests(guests)
    code = gcmc.MOVES.index(kind)
    mols, news, exp = [], [], []
    for i in range(3):
        g = guests[i].reshape(4, 3, 3)
        m = int(rng.integers(0, 4))
        # the molecule whole (atoms unwrapped against atom 0), as the kernel treats it
        whole = g[m][0] + wrapped(g[m] - g[m][0], setup.tril[0])
        if kind == "translate":
            new = wrapped(g[m] + rng.normal(0, 0.5, 3), setup.tril[0])
        elif kind == "rotate":
            from scipy.spatial.transform import Rotation

            c = whole.mean(0)
            R = Rotation.random(random_state=int(rng.integers(1 << 30))).as_matrix()
            new = wrapped((whole - c) @ R.T + c, setup.tril[0])
        elif kind == "reinsert":
            # full random rotation about the centre, then a uniform fractional offset
            from scipy.spatial.transform import Rotation

            c = whole.mean(0)
            R = Rotation.random(random_state=int(rng.integers(1 << 30))).as_matrix()
            new = wrapped((whole - c) @ R.T + c + rng.uniform(0, 1, 3) @ L, setup.tril[0])
        elif kind == "insert":
            new = wrapped(random_molecule(rng, L, mpos), setup.tril[0])
        else:
            new = None
        before = guests[i]
        if kind == "insert":
            after = np.concatenate([before, new])
        elif kind == "delete":
            after = np.concatenate([g[j] for j in range(4) if j != m])
        else:
            gg = g.copy()
            gg[m] = new
            after = gg.reshape(-1, 3)
        mols.append(m)
        news.append(new)
        exp.append(oracle_energy(setup, after) - oracle_energy(setup, before))
    # the GPU moves the guests it holds (float32); the oracle saw float64 copies
    out = mc.evaluate([code] * 3, mols, news)
    got = out[:, 0]
    np.testing.assert_allclose(got, exp, rtol=2e-5, atol=2e-5)


def test_ideal_gas_loading_is_poisson():
    from kups_gb300 import gcmc

    setup = small_setup(n_sys=64, tail=False, charges=False)
    setup.epsilon = np.zeros_like(setup.epsilon)
    setup.max_mol = 40  # Poisson(3) reaches 16 molecules about once in 10^7 system-steps
    vol = abs(np.prod(setup.tril[0, [0, 2, 5]]))
    target = 3.0
    setup.log_activity = np.full(64, np.log(target / vol))
    mc = gcmc.GCMC(setup, seed=11)
    mc.launch(2000)
    samples = []
    for _ in range(120):
        mc.launch(50)
        samples.append(mc.n_mol.cpu().numpy().copy())
    mc.check()
    n = np.array(samples, float)
    mean = n.mean()
    # all systems share the move-kind sequence (as the reference's propose_mixed does), so
    # their loadings are correlated: the standard error comes from the time series of the
    # cross-system mean
    t = n.mean(1)
    se = t.std(ddof=1) / np.sqrt(len(t))
    assert abs(mean - target) < 4 * se, (mean, se)
    st = mc.statistics()
    assert st["insert"][0] > 0 and st["delete"][0] > 0


# ----------------------------------------------------------------------------- learned insertion proposal
def _blob_proposal(seed=0, grid=16):
    from kups_gb300.mlp import LearnedInsertionProposal

    rng = np.random.default_rng(seed)
    c = np.array([[0.2, 0.3, 0.4], [0.7, 0.75, 0.1]])[rng.integers(0, 2, 100000)]
    data = (c + 0.05 * rng.normal(size=c.shape)) % 1.0
    net = LearnedInsertionProposal(seed=seed + 1, grid=grid)
    net.train(torch.as_tensor(data, device="cuda"), steps=200, batch=8192, lr=3e-3)
    net.build_grid()
    return net


def _anchor_frac(pos, tril):
    """Atom mean (unwrapped against atom 0) of float32 positions, fractional, in float64."""
    L = ouc.lattice_from_tril(tril)
    inv = np.linalg.inv(L)
    p = np.asarray(pos, np.float32).astype(np.float64)
    d = (p - p[0]) @ inv
    d -= np.round(d)
    return (p[0] @ inv + d.mean(0)) % 1.0


@pytest.mark.parametrize("kind", ["insert", "delete"])
def test_learned_proposal_log_ratio_matches_oracle(kind):
    """ln acc with the learned density minus ln acc with uniform insertion is -ln q_f(centre)
    for an insertion and +ln q_f(centre) for a deletion (bar: 1e-4 absolute, the float32
    centre of the molecule)."""
    from kups_gb300 import gcmc
    from oracle import mlp as om

    net = _blob_proposal()
    node, cdf = net.node.cpu().numpy(), net.cdf.cpu().numpy()
    setup = small_setup(n_sys=3)
    rng = np.random.default_rng(7)
    L = ouc.lattice_from_tril(setup.tril[0])
    guests = [np.concatenate([wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
                              for _ in range(4)]) for _ in range(3)]
    code = gcmc.MOVES.index(kind)
    mols = [int(m) for m in rng.integers(0, 4, 3)]
    news = [wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0]) if kind == "insert" else None
            for _ in range(3)]
    outs = []
    for proposal in (None, net):
        mc = gcmc.GCMC(setup, seed=5)
        mc.set_guests(guests)
        mc.use_proposal(proposal)
        outs.append(mc.evaluate([code] * 3, mols, news))
    got = outs[1][:, 3] - outs[0][:, 3]
    exp = []
    for i in range(3):
        mol = news[i] if kind == "insert" else guests[i].reshape(4, 3, 3)[mols[i]]
        lq = om.log_q(node, cdf, net.grid, _anchor_frac(mol, setup.tril[0])[None])[0]
        exp.append(-lq if kind == "insert" else lq)
    np.testing.assert_allclose(got, exp, atol=1e-4)
    np.testing.assert_allclose(outs[1][:, 0], outs[0][:, 0], rtol=1e-12)  # same energy change


def test_ideal_gas_with_learned_proposal_stays_uniform_and_poisson():
    """Detailed balance of the learned insertion: without interactions the loading must stay
    Poisson with mean a V and the molecules must fill the cell uniformly, although insertions
    are drawn mostly inside two blobs (2 % of the volume)."""
    from kups_gb300 import gcmc

    net = _blob_proposal(3)
    setup = small_setup(n_sys=64, tail=False, charges=False)
    setup.epsilon = np.zeros_like(setup.epsilon)
    setup.max_mol = 40  # Poisson(3) reaches 16 molecules about once in 10^7 system-steps
    vol = abs(np.prod(setup.tril[0, [0, 2, 5]]))
    target = 3.0
    setup.log_activity = np.full(64, np.log(target / vol))
    mc = gcmc.GCMC(setup, seed=13)
    mc.use_proposal(net)
    mc.launch(2000)
    samples, centres = [], []
    for _ in range(120):
        mc.launch(50)
        samples.append(mc.n_mol.cpu().numpy().copy())
        centres.append(mc.molecule_centres_frac().cpu().numpy())
    mc.check()
    n = np.array(samples, float)
    t = n.mean(1)
    se = t.std(ddof=1) / np.sqrt(len(t))
    assert abs(n.mean() - target) < 4 * se, (n.mean(), se)
    c = np.concatenate(centres)
    blobs = np.array([[0.2, 0.3, 0.4], [0.7, 0.75, 0.1]])
    d = c[:, None, :] - blobs[None]
    d -= np.round(d)
    r = np.sqrt(((d @ ouc.lattice_from_tril(setup.tril[0])) ** 2).sum(-1)).min(1)  # Cartesian distance
    inside = float((r < 2.0).mean())
    expected = 2 * 4 / 3 * np.pi * 2.0**3 / vol
    assert abs(inside - expected) < 0.5 * expected + 0.005, (inside, expected)
    st = mc.statistics()
    assert st["insert"][1] > 100 and st["delete"][1] > 100


def test_learned_proposal_gain_and_loading_in_a_porous_host():
    """The learned insertion proposal trained on the plain sampler's molecule centres gives at
    least 3x the accepted insertions per second of uniform insertion, and both samplers run
    from the same equilibrated state agree on the loading: all replicas pooled within 3
    block-averaged standard errors, each of four pressure groups within 4.

    Host: the porous 2000-atom framework (25 A, 90/90/120 degrees, one channel) with its
    Lennard-Jones well depths halved and no charges, 0.1-1 bar at 298 K, 10 A cutoff (every
    cell width exceeds twice the cutoff: minimum image).  Insertions there fail mostly on
    the host, which is what the proposal learns; the loadings (3-15 molecules) equilibrate
    within the run.  (The full-strength host condenses CO2 in its channel at these
    pressures and equilibrates too slowly for a test.)"""
    from kups_gb300 import workloads
    from kups_gb300.mlp import learned_vs_plain

    setup = workloads.gcmc_co2_framework(n_replicas=1024, replicate=None, rc=10.0, alpha=0.3, eps_scale=0.5,
                                         charge_scale=0.0, p_min_bar=0.1, p_max_bar=1.0, max_mol=64)
    out = learned_vs_plain(setup, plain_steps=4000, snapshots=40, train_steps=1500, equil_steps=4000,
                           prod_steps=10000, block=500, groups=4)
    assert out["insertion_gain"] >= 3.0, out["insertion_gain"]
    # pooled: the standard error comes from the block series of the all-replica mean (all
    # replicas share the move-kind sequence, so their loadings are correlated)
    assert abs(out["loading_all_z"]) < 3.0, (out["plain"], out["learned"])
    assert np.all(np.abs(out["loading_z"]) < 4.0), out["loading_z"]


@pytest.mark.parametrize("kind", ["translate", "insert", "delete"])
def test_reciprocal_delta_on_the_full_host_matches_full_recomputation(kind):
    """On the 8000-atom replicated host (|S(k)| up to ~50, 3336 k vectors) the incremental
    reciprocal-space change of a move (float32 per-k terms, float64 sums) equals the difference
    of two full float64 structure-factor evaluations (kups_ewald_recip) within 2e-5 eV."""
    from kups_gb300 import gcmc, workloads
    from kups_gb300.ewald import ewald_recip

    setup = workloads.gcmc_co2_framework(n_replicas=2, max_mol=32)
    rng = np.random.default_rng({"translate": 1, "insert": 2, "delete": 3}[kind])
    L = ouc.lattice_from_tril(setup.tril[0])
    guests = [np.concatenate([wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
                              for _ in range(12)]) for _ in range(2)]
    mc = gcmc.GCMC(setup, seed=3)
    mc.set_guests(guests)
    mols = [int(m) for m in rng.integers(0, 12, 2)]
    news = []
    afters = []
    for i in range(2):
        g = guests[i].reshape(12, 3, 3)
        if kind == "translate":
            new = wrapped(g[mols[i]] + rng.normal(0, 0.7, 3), setup.tril[0])
            gg = g.copy()
            gg[mols[i]] = new
            after = gg.reshape(-1, 3)
        elif kind == "insert":
            new = wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
            after = np.concatenate([guests[i], new])
        else:
            new = None
            after = np.concatenate([g[j] for j in range(12) if j != mols[i]])
        news.append(new)
        afters.append(after)
    out = mc.evaluate([gcmc.MOVES.index(kind)] * 2, mols, news)

    def e_rec(guest_sets):
        pos, q, off = [], [], [0]
        for gp in guest_sets:
            gp = np.asarray(gp, np.float32).astype(np.float64)  # the positions the kernel holds
            pos.append(np.concatenate([setup.fw_positions, gp]))
            q.append(np.concatenate([setup.fw_charges, np.tile(setup.motif_charges, len(gp) // 3)]))
            off.append(off[-1] + len(pos[-1]))
        P = torch.as_tensor(np.concatenate(pos), device="cuda")
        Q = torch.as_tensor(np.concatenate(q), device="cuda")
        O = torch.as_tensor(np.array(off, np.int32), device="cuda")
        e, _, _, _, _ = ewald_recip(P, Q, O, int(np.diff(off).max()), mc.tril, mc.kn, mc.alpha, grad_tril=False)
        return e.cpu().numpy()

    np.testing.assert_allclose(out[:, 2], e_rec(afters) - e_rec(guests), atol=2e-5)


@pytest.mark.parametrize("kind", ["translate", "rotate", "insert", "delete"])
def test_host_group_skipping_changes_nothing(kind):
    """Skipping 32-atom host groups beyond the cutoff leaves every move's energy change
    bit-identical (a skipped group's pairs all lie outside the cutoff and add exactly 0.0)
    on the 8000-atom replicated host."""
    from kups_gb300 import gcmc, workloads

    setup = workloads.gcmc_co2_framework(n_replicas=4, max_mol=32)
    rng = np.random.default_rng({"translate": 5, "rotate": 6, "insert": 7, "delete": 8}[kind])
    L = ouc.lattice_from_tril(setup.tril[0])
    guests = [np.concatenate([wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
                              for _ in range(10)]) for _ in range(4)]
    mols = [int(m) for m in rng.integers(0, 10, 4)]
    news = []
    for i in range(4):
        g = guests[i].reshape(10, 3, 3)
        if kind == "translate":
            news.append(wrapped(g[mols[i]] + rng.normal(0, 1.0, 3), setup.tril[0]))
        elif kind == "rotate":
            from scipy.spatial.transform import Rotation

            c = g[mols[i]].mean(0)
            R = Rotation.random(random_state=int(rng.integers(1 << 30))).as_matrix()
            news.append(wrapped((g[mols[i]] - c) @ R.T + c, setup.tril[0]))
        elif kind == "insert":
            news.append(wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0]))
        else:
            news.append(None)
    outs = []
    for use_groups in (True, False):
        mc = gcmc.GCMC(setup, seed=3)
        mc.set_guests(guests)
        if not use_groups:
            mc.fw_group = None
        outs.append(mc.evaluate([gcmc.MOVES.index(kind)] * 4, mols, news))
    np.testing.assert_array_equal(outs[0], outs[1])
    assert np.all(np.isfinite(outs[0]))


# ----------------------------------------------------------------------------- device observables
def test_device_block_sums_equal_the_per_step_series():
    """kups_gcmc_run's per-step U, N, U N, N^2, U^2 sums equal, bit for bit, the sums of the
    per-step series read after one-step launches of an identical sampler (same seed: the step
    counter keys the random numbers, so launch length does not change the trajectory); the
    block analysis equals the oracle's analysis of that series (application/mcmc/analysis.py)."""
    from kups_gb300 import gcmc
    from oracle import analysis as oan

    setup = small_setup(n_sys=4, seed=2)
    setup.log_activity = np.full(4, -6.0)
    a, b = gcmc.GCMC(setup, seed=5), gcmc.GCMC(setup, seed=5)
    block, nb = 20, 6
    u_series, n_series = [], []
    for _ in range(block * nb):
        a.launch(1)
        u_series.append(a.energy.cpu().numpy().copy())
        n_series.append(a.n_mol.cpu().numpy().astype(float))
    a.check()
    sums = b.run_blocks(nb, block)
    u, n = np.array(u_series), np.array(n_series)
    assert n.max() > 0 and np.ptp(n) > 0
    for k in range(nb):
        exp = np.zeros((4, 5))
        for t in range(k * block, (k + 1) * block):
            for s in range(4):
                exp[s] += [u[t, s], n[t, s], u[t, s] * n[t, s], n[t, s] * n[t, s], u[t, s] * u[t, s]]
        np.testing.assert_array_equal(sums[k], exp)
    res = b.analyze(sums, block, n_blocks=3)
    for s in range(4):
        ref = oan.analyze_single_system(u[:, s], n[:, s], setup.temperature[s], 3)
        np.testing.assert_allclose(res["energy"].mean[s], ref["energy"][0], rtol=1e-12)
        np.testing.assert_allclose(res["loading"].mean[s], ref["loading"][0][0], rtol=1e-12)
        if np.isfinite(ref["heat_of_adsorption"][0][0]):
            np.testing.assert_allclose(res["heat_of_adsorption"].mean[s], ref["heat_of_adsorption"][0][0],
                                       rtol=1e-9)


def test_guest_stress_is_the_volume_derivative_of_the_guest_energy():
    """GCMC.guest_stress (mcmc_rigid.py:385-436) on molecules that straddle the cell faces:
    Tr(potential) / 3 equals -dU/dV of the guest-only energy (LJ + Ewald with the intramolecular
    exclusion + LJ tail) when the cell scales and every molecule moves rigidly with its centre
    (central differences, relative step 1e-6); the potential part is the oracle's molecular
    virial stress of the same gradients; the tail and ideal-gas parts are the oracle's formulas."""
    from kups_gb300 import gcmc
    from oracle import lennard_jones as olj
    from oracle import observables as oobs

    setup = small_setup(n_sys=2, rc=5.0)
    L = ouc.lattice_from_tril(setup.tril[0])
    rng = np.random.default_rng(21)
    mpos = co2_template()[0]
    guests = [wrapped(np.concatenate([random_molecule(rng, L, mpos) for _ in range(n)]), setup.tril[0])
              for n in (7, 5)]
    mc = gcmc.GCMC(setup, seed=1)
    mc.set_guests(guests)
    res = {k: v.cpu().numpy() for k, v in mc.guest_stress().items()}
    pos, q, sp, sysi, grp = mc.guest_table()
    _, g, gt = mc.guest_potential(pos, q, sp, sysi, grp)
    p, s, gr = pos.cpu().numpy(), sysi.cpu().numpy(), grp.cpu().numpy()
    G = int(gr.max()) + 1
    mol = oobs.molecular_virial_stress(p, g.cpu().numpy(), s, gr, G, setup.tril, gt.cpu().numpy())
    scale = np.abs(mol).max()
    np.testing.assert_allclose(res["potential"], mol, rtol=0, atol=1e-10 * scale)

    com, _ = oobs.group_centres(p, gr, G, s, setup.tril)
    w = p - ouc.wrap(p - com[gr], setup.tril[s])

    def energy(eps):
        pe = torch.as_tensor(p + eps * w, device="cuda")
        return mc.guest_potential(pe, q, sp, sysi, grp, tril=setup.tril * (1 + eps))[0].cpu().numpy()

    h = 1e-6
    dU = (energy(h) - energy(-h)) / (2 * h)
    p_fd = -dU / (3 * ouc.volume(setup.tril))
    p_virial = np.trace(res["potential"], axis1=1, axis2=2) / 3
    np.testing.assert_allclose(p_virial, p_fd, rtol=0, atol=1e-5 * scale)

    counts = np.zeros((2, setup.sigma.shape[0]))
    for i, n in enumerate((7, 5)):
        np.add.at(counts[i], setup.fw_species, 1)
        np.add.at(counts[i], np.tile(setup.motif_species, n), 1)
    pt = olj.tail_correction_pressure(counts, setup.tril, setup.sigma, setup.epsilon, setup.rc_lj,
                                      setup.epsilon > 0)
    np.testing.assert_allclose(res["tail_correction"], pt[:, None, None] * np.eye(3), rtol=1e-10, atol=1e-300)
    pi = oobs.ideal_gas_pressure([7, 5], setup.temperature, setup.tril)
    np.testing.assert_allclose(res["ideal_gas"], pi[:, None, None] * np.eye(3), rtol=1e-12, atol=1e-300)


def test_host_energy_cache_hit_equals_the_recomputed_value():
    """Minimum-image path with the host energy cache (kups_gcmc_args.host_cache): a move whose
    old molecule misses computes both ends against the host and stores the old one; the same
    move again reads it back and gives the same energy change bit for bit; the uncached kernel
    agrees within the float32 pair sums' rounding.  Entries follow their molecules on deletion."""
    from kups_gb300 import gcmc
    from oracle import unitcell as ouc

    S = 3
    setup = small_setup(n_sys=S, rc=5.0)
    L = ouc.lattice_from_tril(setup.tril[0])
    rng = np.random.default_rng(4)
    guests = [np.concatenate([wrapped(random_molecule(rng, L, setup.motif_positions), setup.tril[0])
                              for _ in range(5)]) for _ in range(S)]
    mc = gcmc.GCMC(setup, seed=2)
    mc.set_guests(guests)
    off = mc.clone()
    off.use_host_cache = False
    kinds, mols = np.full(S, 4), np.full(S, 1)  # delete molecule 1 (rejected: nothing changes)
    assert float(mc.host_cache[:, 1, 1].abs().max()) == 0.0
    first = mc.evaluate(kinds, mols, [None] * S)
    assert bool((mc.host_cache[:, 1, 1] != 0).all())  # the miss stored the old end
    second = mc.evaluate(kinds, mols, [None] * S)
    np.testing.assert_array_equal(first, second)
    plain = off.evaluate(kinds, mols, [None] * S)
    np.testing.assert_allclose(first[:, :3], plain[:, :3], rtol=1e-6, atol=1e-6)
    # a translation of molecule 2: the old end from a filled entry, the new end computed
    apm = len(setup.motif_charges)
    moved = [wrapped(guests[s].reshape(-1, apm, 3)[2] + 0.3, setup.tril[0]) for s in range(S)]
    mc.evaluate(np.full(S, 4), np.full(S, 2), [None] * S)  # fill molecule 2's entry
    a = mc.evaluate(np.zeros(S, int), np.full(S, 2), moved)
    b = off.evaluate(np.zeros(S, int), np.full(S, 2), moved)
    np.testing.assert_allclose(a[:, :3], b[:, :3], rtol=1e-6, atol=1e-6)
    # free-running steps from a relaxed state (the random start overlaps): the sum of the
    # accepted changes against E(after) - E(before); a wrong cached host energy would be off by
    # a molecule's host energy (tenths of an eV)
    mc.launch(400)
    mc.check()
    start = mc.guest_positions()
    mc.energy.zero_()
    mc.launch(400)
    mc.check()
    got = mc.energy.cpu().numpy()
    state = mc.guest_positions()
    for s in range(S):
        e0 = oracle_energy(setup, start[s].astype(np.float64).reshape(-1, 3))
        e1 = oracle_energy(setup, state[s].astype(np.float64).reshape(-1, 3))
        assert abs(e0) < 1e3, e0  # relaxed
        assert abs((e1 - e0) - got[s]) < 2e-3, (s, e0, e1 - e0, got[s])
    assert int(mc.accepted.sum()) > 50
