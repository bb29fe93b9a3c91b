"""The reference's statistical anchors, run on the GPU kernels.

The reference validates its MD and GCMC applications by runs whose means must lie within
10 standard errors of stored expectations (ci/statistical/validate.py:30, 49-80; expected
values in ci/statistical/expected/*.yaml, inputs in ci/statistical/inputs/**).  The fixtures
(tests/golden/make_statistical_fixtures.py) carry those inputs and expectations; the runs here
use this library's own random streams, so the comparison is statistical, with the reference's
bar |mean - expected| < 10 sigma_expected.

* Argon NVT (md_nvt_lj_argon): 256 Ar from argon_fcc.cif (21.04 A cube), LJ sigma 3.405 A,
  eps 0.0103236 eV, cutoff 10 A, no tail correction, BAOAB dt 2 fs, friction 1 / fs (the input's
  friction_coefficient is per fs: application/md/data.py:200-201), 100 K;
  5000 warm-up steps, 20000 production steps on the fused kernel: potential, kinetic and total
  energy, temperature (3N - 3 degrees of freedom) and the reference's pressure statistic
  (-Tr(dE/dL) / 3V, lattice gradient at fixed Cartesian positions).
* CO2 GCMC in RUBTAK (gcmc_co2_rubtak): the DDEC-charged host replicated 2 x 2 x 2, TraPPE CO2,
  LJ cutoff 12 A with tail correction, Ewald real cutoff 12 A at precision 1e-6, 10 kPa,
  298.15 K (Peng-Robinson fugacity), translate / rotate / reinsert / exchange at 1:1:1:2;
  1000 warm-up and 5000 production cycles of 20 steps, on 32 independent replicas:
  loading and heat of adsorption.
"""

import json
import math
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _expected(name):
    with open(os.path.join(GOLDEN, "statistical_expected.json")) as f:
        d = json.load(f)
    return d[name], d["tolerance_sigmas"]


def _check(name, value, expected, tol):
    mean, sem = expected
    z = abs(value - mean) / sem
    print(f"{name}: {value:.6g} (expected {mean:.6g} +- {sem:.3g}, |diff| = {z:.2f} sigma)")
    assert z < tol, (name, value, mean, sem, z)
    return z


def test_argon_nvt_matches_the_reference_statistics():
    from kups_gb300 import md, potential
    from kups_gb300.units import BOLTZMANN_CONSTANT, FEMTO_SECOND
    from oracle.unitcell import lattice_from_lengths_angles, tril_from_lattice

    ref, tol = _expected("md_nvt_lj_argon")
    st = ref["settings"]
    fx = np.load(os.path.join(GOLDEN, "argon_fcc.npz"))
    L = lattice_from_lengths_angles(fx["lengths"], fx["angles"])
    tril = tril_from_lattice(L)[None]
    pos = fx["frac"] @ L
    n = len(pos)
    mass = np.full(n, 39.948)
    rng = np.random.default_rng(42)
    T = st["temperature_k"]
    mom = rng.normal(size=(n, 3)) * np.sqrt(mass * T * BOLTZMANN_CONSTANT)[:, None]
    mom -= mass[:, None] * (mom.sum(0) / mass.sum())  # no centre-of-mass drift
    c = lambda x, dt=torch.float64: torch.as_tensor(np.asarray(x), dtype=dt).cuda()
    prm = potential.LennardJonesParameters(("Ar",), torch.tensor([[st["sigma_a"]]]), torch.tensor([[st["epsilon_ev"]]]),
                                           torch.tensor([st["cutoff_a"]], dtype=torch.float64))
    state = md.MDState(md.MDParticles(c(pos), c(mom), c(mass), c(np.zeros(n), torch.int32), c(np.zeros(n), torch.int32)),
                       md.MDSystems(c(tril), c([st["time_step_fs"] * FEMTO_SECOND]), c([T]),
                                    c([st["friction_per_fs"] / FEMTO_SECOND])),
                       prm, skin=1.0)
    prop = md.make_baoab_langevin_step()
    packed = md.pack(state)
    prop.run_packed(packed, st["warmup_steps"], seed=42, step0=0)
    steps, chunk = 20000, 10
    pe = torch.zeros((steps, 1), dtype=torch.float64, device="cuda")
    ke = torch.zeros_like(pe)
    vir = torch.zeros((steps, 1, 6), dtype=torch.float64, device="cuda")
    phys = torch.zeros(steps // chunk, dtype=torch.float64, device="cuda")
    step0 = st["warmup_steps"]
    for k in range(steps // chunk):
        sl = slice(k * chunk, (k + 1) * chunk)
        prop.launch(packed, chunk, seed=42, step0=step0, trace_pe=pe[sl], trace_ke=ke[sl], trace_virial=vir[sl])
        phys[k] = packed.pressure[0]
        step0 += chunk
    torch.cuda.synchronize()
    pe, ke, vir = pe.cpu().numpy()[:, 0], ke.cpu().numpy()[:, 0], vir.cpu().numpy()[:, 0]
    temp = 2.0 * ke / ((3 * n - 3) * BOLTZMANN_CONSTANT)
    # The reference's logged "pressure" is Tr(stress) / 3 with stress = -dE/dL / V, dE/dL the
    # potential's lattice gradient at fixed Cartesian positions (application/md/data.py:102-107,
    # application/md/analysis.py:101): no kinetic part, and the positions wrapped into
    # [-0.5, 0.5) as both codes wrap them.  The per-step dE/dtril trace is that gradient.
    vol = abs(np.prod(tril[0, [0, 2, 5]]))
    prs = -(vir[:, 0] + vir[:, 2] + vir[:, 5]) / (3.0 * vol)
    print(f"physical pressure (2K - Tr W) / 3V: {phys.mean().item():.4g} eV/A^3 (not a reference statistic)")
    exp = ref["expected"]
    zs = [_check("potential_energy", pe.mean(), exp["potential_energy"], tol),
          _check("kinetic_energy", ke.mean(), exp["kinetic_energy"], tol),
          _check("total_energy", (pe + ke).mean(), exp["total_energy"], tol),
          _check("temperature", temp.mean(), exp["temperature"], tol),
          _check("pressure", prs.mean(), exp["pressure"], tol)]
    # this run's own standard errors (20 blocks) are of the reference's size
    sem = lambda x: np.array_split(x, 20)
    own = np.std([b.mean() for b in sem(pe)], ddof=1) / math.sqrt(20)
    assert own < 5 * exp["potential_energy"][1], own
    assert max(zs) < tol


def test_gcmc_co2_in_rubtak_matches_the_reference_statistics():
    from kups_gb300 import gcmc, workloads
    from kups_gb300.ewald import estimate_ewald_parameters, kvecs_from_kmax
    from kups_gb300.units import BOLTZMANN_CONSTANT, PASCAL
    from oracle.unitcell import lattice_from_lengths_angles, tril_from_lattice

    ref, tol = _expected("gcmc_co2_rubtak")
    st = ref["settings"]
    fx = np.load(os.path.join(GOLDEN, "rubtak.npz"))
    L = lattice_from_lengths_angles(fx["lengths"], fx["angles"])
    tril1 = tril_from_lattice(L)
    r = st["replication"]
    fw, tril = workloads.replicate_host(fx["frac"] @ L, tril1, (r, r, r))
    k = r**3
    fw_sp, fw_q = np.tile(fx["species"], k), np.tile(fx["charges"], k)
    n_sp = len(fx["sigma"])
    sig = np.concatenate([fx["sigma"], fx["co2_sigma"]])
    eps = np.concatenate([fx["epsilon"], fx["co2_epsilon"]])
    sigma, epsilon = gcmc.lorentz_berthelot(sig, eps)
    rc = st["cutoff_a"]
    ew = estimate_ewald_parameters(fw_q, tril, real_cutoff=rc, epsilon_total=st["ewald_precision"])
    kn = kvecs_from_kmax(tril, ew["k_max"])
    T, p = st["temperature_k"], st["pressure_pa"]
    kT = T * BOLTZMANN_CONSTANT
    lnf = gcmc.peng_robinson_log_fugacity(p, T, st["critical_pressure_pa"], st["critical_temperature_k"],
                                          st["acentric_factor"]).log_fugacity[0]
    la = lnf + math.log(PASCAL) - math.log(kT)
    R = 32
    setup = gcmc.GCMCSetup(
        fw_positions=fw, fw_species=fw_sp, fw_charges=fw_q, fw_start=np.zeros(R, int), fw_count=np.full(R, len(fw)),
        tril=np.repeat(tril[None], R, 0), motif_positions=np.array(st["co2_positions"], float),
        motif_species=np.array([n_sp, n_sp + 1, n_sp + 1]), motif_charges=np.array(st["co2_charges"]),
        sigma=sigma, epsilon=epsilon, rc_lj=np.full(R, rc), rc_ew=np.full(R, rc), alpha=np.full(R, ew["alpha"]),
        kvec_n=np.repeat(kn[None], R, 0), temperature=np.full(R, T), log_activity=np.full(R, la),
        max_mol=st["max_num_adsorbates"], tail_correction=st["tail_correction"])
    mc = gcmc.GCMC(setup, seed=42)
    cyc = st["min_cycle_length"]
    mc.launch(st["warmup_cycles"] * cyc)
    block = 50 * cyc
    sums = mc.run_blocks(st["cycles"] * cyc // block, block)  # [blocks, R, 5]
    tot = sums.sum(0) / (sums.shape[0] * block)  # per replica <U>, <N>, <UN>, <N^2>, <U^2>
    loading = tot[:, 1]
    q = (tot[:, 2] - tot[:, 0] * tot[:, 1]) / (tot[:, 3] - tot[:, 1] ** 2) - kT
    exp = ref["expected"]
    _check("loading", loading.mean(), exp["loading"], tol)
    _check("heat_of_adsorption", q.mean(), exp["heat_of_adsorption"], tol)
    # independent replicas: the spread of their means is of the reference's single-run size
    assert loading.std(ddof=1) < 10 * exp["loading"][1] * math.sqrt(2)
