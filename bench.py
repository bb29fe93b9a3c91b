"""Benchmark of the batched Lennard-Jones MD hot path (atom-steps/s).

Workload (default): 4096 independent cubic argon systems, atom counts
~U{64..2048} (about 4.36 M atoms), reduced densities ~U[0.7, 0.9], per-system
temperatures ~U[80, 140] K, cutoff 2.5 sigma (+0.3 sigma Verlet skin),
BAOAB Langevin (dt 2 fs, friction 1/ps), float32 pair arithmetic with float64
per-system reductions.  Seeded synthetic positions (a jittered lattice subset
with a 0.9 sigma minimum separation).

One bench step = one MD step of every system.  `value` times the fused
persistent kernel on device-resident inputs; `e2e` times the public
propagator API (``FusedLennardJonesMD.__call__``) fed from pinned host
buffers, host<->device copies included; the CPU baseline is the float64
NumPy restatement of the reference's algorithm (dense neighbour list rebuilt
every step, as the reference's MD app does) on a bounded sample of systems.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_STATE = 64  # float4 position+species and float4 momentum+mass, read and written
BYTES_PER_HALF_NEIGHBOUR = 4  # uint16 index, stored for both directions


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--chunk", type=int, default=500, help="MD steps per persistent launch")
    ap.add_argument("--e2e-chunk", type=int, default=50, help="MD steps per public-API call in the e2e leg")
    ap.add_argument("--e2e-calls", type=int, default=4)
    ap.add_argument("--e2e-runs", type=int, default=4,
                    help="runs of whole systems whose host copies overlap the other runs' launches in the e2e leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-gcmc", action="store_true", help="skip the GCMC plain / learned-proposal section")
    ap.add_argument("--no-ewald", action="store_true", help="skip the LJ + Ewald MD (ionic melt) section")
    ap.add_argument("--no-ensembles", action="store_true", help="skip the BAOAB / CSVR / NPT comparison")
    ap.add_argument("--no-autotune", action="store_true", help="library-default launch shape for the MD kernel")
    ap.add_argument("--no-bonded", action="store_true", help="skip the bonded-term (evaluation and MC energy change), "
                    "virial-observable and local-MLIAP timings")
    ap.add_argument("--gcmc-replicas", type=int, default=1024)
    ap.add_argument("--gcmc-equil", type=int, default=100000,
                    help="GCMC equilibration steps (learned proposal) before the plain / learned production runs")
    ap.add_argument("--gcmc-prod", type=int, default=20000, help="GCMC production steps of each sampler")
    ap.add_argument("--no-nve-check", dest="nve_check", action="store_false",
                    help="skip the NVE energy-conservation runs of the LJ + Ewald section")
    ap.add_argument("--strong", action="store_true",
                    help="split one --systems batch across the ranks (cost-balanced contiguous ranges) "
                         "instead of giving every rank its own batch")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(n_systems, seed):
    from kups_gb300 import workloads

    return workloads.batched_uneven_lj(n_systems=n_systems, seed=seed)


def algorithmic_bytes_per_step(W) -> float:
    """64 B of state per atom-step plus 4 B per half-list neighbour within rc + skin."""
    counts = np.bincount(W.system, minlength=W.n_systems).astype(np.float64)
    vol = W.tril[:, 0] * W.tril[:, 2] * W.tril[:, 5]
    rl = W.cutoff + W.skin
    n_half = 2.0 / 3.0 * math.pi * rl**3 * counts / vol
    return float(np.sum(counts * (BYTES_STATE + BYTES_PER_HALF_NEIGHBOUR * n_half)))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nme, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nme)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def read_profile_value(key):
    """A per-atom-step figure of the MD kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "md_lj_batched_uneven_ncu.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            return float(line.split(":")[1].split()[0])
    return None


def read_traffic():
    """DRAM bytes per atom-step of the MD kernel from the committed ncu summary, if present."""
    return read_profile_value("dram_bytes_per_atom_step")


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- CPU legs
def _cpu_sample_worker(args):
    """Runs BAOAB steps of the float64 oracle on a few systems until the budget is spent."""
    sys_ids, seconds, n_systems = args
    sys.path.insert(0, ROOT)
    from oracle import md as omd

    W = workload(n_systems, 1)
    rng = np.random.default_rng(0)
    done = 0
    t0 = time.perf_counter()
    for s in sys_ids:
        m = W.system == s
        pos = W.positions[m]
        n = pos.shape[0]
        args_ = (W.masses[m], np.zeros(n, int), W.species[m], W.tril[s:s + 1], W.sigma, W.epsilon, [W.cutoff])
        e, f, _ = omd.lj_forces(pos, np.zeros(n, int), W.species[m], W.tril[s:s + 1], W.sigma, W.epsilon, [W.cutoff])
        mom = W.momenta[m]
        while time.perf_counter() - t0 < seconds:
            noise = rng.standard_normal((1, n, 3))
            pos, mom, f, _ = omd.baoab(pos, mom, f, W.masses[m], np.zeros(n, int), W.species[m], W.tril[s:s + 1],
                                       W.sigma, W.epsilon, [W.cutoff], W.time_step[s:s + 1], W.temperature[s:s + 1],
                                       W.friction[s:s + 1], noise)
            done += n
            if done >= 3 * n * 4:  # a few steps per system, then the next system
                break
        if time.perf_counter() - t0 >= seconds:
            break
    return done, time.perf_counter() - t0


def cpu_baseline(n_systems, seconds, processes):
    """Atom-steps/s of the oracle on a sample of the workload's systems."""
    rng = np.random.default_rng(123)
    pick = rng.choice(n_systems, size=64, replace=False).tolist()
    if processes <= 1:
        done, el = _cpu_sample_worker((pick, seconds, n_systems))
        return done / el, 1, f"{done} atom-steps of BAOAB over sampled systems in {el:.1f} s"
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    chunks = [pick[i::processes] for i in range(processes)]
    t0 = time.perf_counter()
    with ctx.Pool(processes) as pool:
        res = pool.map(_cpu_sample_worker, [(c, seconds, n_systems) for c in chunks])
    el = time.perf_counter() - t0
    done = sum(r[0] for r in res)
    rate = sum(r[0] / r[1] for r in res)
    return rate, processes, f"{done} atom-steps of BAOAB over sampled systems on {processes} processes in {el:.1f} s"


# ----------------------------------------------------------------------------- GPU leg
def run_ours(a):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    from kups_gb300 import md

    if a.strong:
        from kups_gb300.sharding import rank_systems

        W = workload(a.systems, 1)
        lo, hi = rank_systems(np.bincount(W.system, minlength=W.n_systems), rank, world)
        W = W.subset(lo, hi)
    else:
        W = workload(a.systems, 1 + rank)
    state = state_from_workload(W, torch)
    prop = md.make_baoab_langevin_step()
    packed = md.pack(state)
    tuned = None
    if not a.no_autotune:
        from kups_gb300.autotune import autotune_md

        # launch shape picked on a copy of the state (restored after every trial); untimed
        tuned = autotune_md(prop, packed)
    a.tuned = (prop.block_threads, prop.min_lanes_per_atom)
    # warm-up (includes the first list build and force evaluation)
    prop.run_packed(packed, max(a.warmup, 3), seed=11, step0=0)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    chunks = []
    k = a.steps
    while k > 0:
        chunks.append(min(a.chunk, k))
        k -= chunks[-1]
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in chunks]
    status = torch.zeros(3, device="cuda", dtype=torch.int64)
    status[2] = -1
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    step0 = max(a.warmup, 3)
    for (e0, e1), c in zip(events, chunks):
        e0.record(stream)
        prop.launch(packed, c, seed=11, step0=step0, status=status, virial=False)
        e1.record(stream)
        step0 += c
    t_end.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    from kups_gb300.neighborlist import read_status
    from kups_gb300 import _lib

    _lib.raise_status(read_status(status))
    ms = t_start.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    if world > 1:
        n_all = torch.tensor([W.n_atoms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(n_all)
        atom_steps = float(n_all.item()) * a.steps
    else:
        atom_steps = W.n_atoms * a.steps
    value = atom_steps / (ms / 1e3)
    launch_ms = [e0.elapsed_time(e1) for e0, e1 in events]
    bytes_step = algorithmic_bytes_per_step(W)
    achieved = sum(bytes_step * c for c in chunks) / (sum(launch_ms) / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic_per_atom_step = read_traffic()
    line = {
        "metric": "batched LJ MD atom-steps/s",
        "value": value,
        "unit": "atom-steps/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": max(a.warmup, 3),
        "ms_per_step": ms / a.steps,
        "higher_is_better": True,
        "scaling": "strong" if a.strong else "weak",
        "vs_baseline": None,
        "dtype": "fp32 pair / fp64 sums",
        "data": "synthetic (seeded)",
        "config": {
            "workload": f"batched uneven LJ MD: {W.n_systems} systems, N~U[64,2048] ({W.n_atoms} atoms), "
                        f"rho*~U[0.7,0.9], T~U[80,140] K, rc 2.5 sigma + 0.3 sigma skin, BAOAB dt 2 fs",
            "systems_per_gpu": W.n_systems,
            "atoms_per_gpu": W.n_atoms,
            "steps_per_launch": chunks[0],
            "launch_shape": {"block_threads": prop.block_threads or 1024,
                             "min_lanes_per_atom": prop.min_lanes_per_atom or 2,
                             "chosen_by": "kups_gb300.autotune.autotune_md" if tuned else "library default",
                             "candidates_ms_per_step": ([[bt, ml, ms] for bt, ml, ms in tuned.table]
                                                        if tuned else None)},
            "l2": "inputs larger than L2 (state 4.4M atoms x 48 B + Verlet lists)",
            "parallelism": (f"systems split over {world} ranks by cost (contiguous ranges), no collective"
                            if a.strong else f"replicas x{world} (independent systems, no collective)"),
        },
        "gpu_launches": len(chunks),
        "roofline": {
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": (traffic_per_atom_step * W.n_atoms * chunks[0]) if traffic_per_atom_step else None,
            "peak_source": peak_kind,
            "algorithmic_bytes_per_atom_step": bytes_step / W.n_atoms,
        },
        "clocks": clk,
    }
    # FP32 pipe: 30 flop per pair within the cutoff counted once (half list), n_half from each
    # system's density; peak derived as SMs x 128 FP32 lanes x 2 flop x SM clock under load
    counts = np.bincount(W.system, minlength=W.n_systems).astype(float)
    vol = np.abs(W.tril[:, 0] * W.tril[:, 2] * W.tril[:, 5])
    n_half = (4.0 / 3.0) * math.pi * W.cutoff**3 * (counts / vol) / 2.0
    flop_atom_step = 30.0 * float((n_half * counts).sum() / counts.sum())
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    fp32_achieved = value * flop_atom_step / 1e12 / max(world, 1)
    line["fp32_roofline"] = {"achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": fp32_achieved / fp32_peak, "flop_per_atom_step": flop_atom_step,
                             "peak_source": f"derived: {sms} SMs x 128 FP32 lanes x 2 flop x {mhz:.0f} MHz"}
    # shared memory: the kernel keeps every system on chip, so its on-chip ceiling is the
    # shared-memory data path (one wavefront per clock per SM); wavefronts per atom-step from the
    # committed ncu capture of the same kernel and workload
    wf = read_profile_value("shared_wavefronts_per_atom_step")
    if wf is not None:
        smem_peak = sms * mhz * 1e6
        smem_achieved = value * wf / max(world, 1)
        line["smem_roofline"] = {"achieved": smem_achieved, "peak": smem_peak, "unit": "wavefronts/s",
                                 "frac": smem_achieved / smem_peak, "wavefronts_per_atom_step": wf,
                                 "bank_conflict_share": read_profile_value("shared_bank_conflict_share"),
                                 "peak_source": f"derived: {sms} SMs x 1 shared-memory wavefront per clock x {mhz:.0f} MHz",
                                 "source": "profiles/md_lj_batched_uneven_ncu.txt"}
    line["steady_state"] = steady_state(prop, packed, torch, step0, W.n_atoms)
    if not a.no_e2e:
        line["e2e"] = run_e2e(a, W, torch)
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        rate, cores, sample = cpu_baseline(a.systems, a.cpu_seconds, 1)
        line["cpu_baseline"] = {"value": rate, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                                "sample": sample}
    if rank == 0 and not a.no_ensembles:
        line["ensembles"] = run_ensembles(a, W, torch)
    if rank == 0 and not a.no_ewald:
        line["argon_nvt"] = run_argon(a, torch)
        line["lj_ewald_md"] = run_ewald_md(a)
    if rank == 0 and not a.no_bonded:
        line["bonded"] = run_bonded(a)
        line["local_mliap"] = run_mliap(a)
        line["virial_observables"] = run_observables(a)
    if rank == 0 and not a.no_gcmc:
        line["gcmc"] = run_gcmc(a)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def steady_state(prop, packed, torch, step0, n_atoms, steps=500, traced=100):
    """After the timed region: one launch of `steps` steps (list builds at their natural rate,
    every Verlet list past its first use) and one launch of `traced` steps that also records the
    potential and kinetic energy and dE/dtril of every system after every step (the reference's
    potential returns energy and cell gradient at every step), each device-timed."""
    from kups_gb300 import _lib
    from kups_gb300.neighborlist import read_status

    out = {}
    for tag, n, tr in (("ms_per_step", steps, False), ("ms_per_step_with_energy_and_virial", traced, True)):
        S = packed.n_systems
        tpe = torch.zeros((n, S), dtype=torch.float64, device="cuda") if tr else None
        tke = torch.zeros((n, S), dtype=torch.float64, device="cuda") if tr else None
        tvir = torch.zeros((n, S, 6), dtype=torch.float64, device="cuda") if tr else None
        packed.rebuilds = torch.zeros(S, dtype=torch.int32, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        st = prop.launch(packed, n, seed=11, step0=step0, virial=False, trace_pe=tpe, trace_ke=tke,
                         trace_virial=tvir)
        e1.record()
        torch.cuda.synchronize()
        _lib.raise_status(read_status(st))
        step0 += n
        out[tag] = e0.elapsed_time(e1) / n
        if not tr:
            out["atom_steps_per_s"] = n_atoms / (out[tag] / 1e3)
            out["list_builds_per_system_per_100_steps"] = float(packed.rebuilds.double().mean()) * 100.0 / n
        packed.rebuilds = None
    out["steps"] = steps
    out["traced_steps"] = traced
    return out


def run_ensembles(a, W, torch, steps=200):
    """The same batched workload under each thermostat / barostat of the fused kernel, one
    persistent launch of `steps` steps each after 10 warm-up steps: BAOAB, CSVR (tau_T 100 fs)
    and CSVR + stochastic cell rescaling (P0 1 bar, tau_P 1 ps, beta 2e-4 / bar, mu within
    [0.99, 1 / 0.99]; two force evaluations per step, as the reference's NPT step does)."""
    from kups_gb300 import md
    from kups_gb300.units import FEMTO_SECOND

    bar = 6.241509074e-7  # eV / A^3
    out = {"workload": "the headline batched workload", "steps_per_launch": steps, "ms_per_step": {},
           "atom_steps_per_s": {}}
    for name, make in (("baoab", md.make_baoab_langevin_step), ("csvr", md.make_csvr_step),
                       ("csvr_npt", md.make_csvr_npt_step)):
        state = state_from_workload(W, torch)
        S = W.n_systems
        full = lambda v: torch.full((S,), float(v), dtype=torch.float64, device="cuda")
        state.systems.thermostat_time_constant = full(100 * FEMTO_SECOND)
        state.systems.target_pressure = full(bar)
        state.systems.pressure_coupling_time = full(1000 * FEMTO_SECOND)
        state.systems.compressibility = full(2e-4 / bar)
        state.systems.minimum_scale_factor = full(0.99)
        prop = make()
        prop.block_threads, prop.min_lanes_per_atom = getattr(a, "tuned", (0, 0))
        packed = md.pack(state)
        prop.run_packed(packed, 10, seed=5, step0=0)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        st = prop.launch(packed, steps, seed=5, step0=10, virial=False)
        t1.record()
        torch.cuda.synchronize()
        from kups_gb300 import _lib
        from kups_gb300.neighborlist import read_status

        _lib.raise_status(read_status(st))
        ms = t0.elapsed_time(t1) / steps
        out["ms_per_step"][name] = ms
        out["atom_steps_per_s"][name] = W.n_atoms / (ms / 1e3)
        del packed, prop
    return out


def _chains(n_systems=2048, n_per=256, seed=7):
    """Seeded chain molecules: a random walk of 1.5 A steps per system in a 40 A cube."""
    rng = np.random.default_rng(seed)
    steps = rng.normal(size=(n_systems, n_per, 3))
    steps *= 1.5 / np.linalg.norm(steps, axis=-1, keepdims=True)
    pos = np.cumsum(steps, axis=1) + rng.uniform(0, 40, (n_systems, 1, 3))
    return pos.reshape(-1, 3), np.repeat(np.arange(n_systems), n_per), n_per


def run_bonded(a, reps=20):
    """Bonded terms on 2048 chain molecules of 256 atoms (524 288 atoms): harmonic bonds, harmonic
    angles, dihedrals and inversions along each chain (about 5.2e5 edges of each kind), two
    species, one kups_bonded_edges launch per kind, summed into one energy / gradient / cell-
    gradient buffer.  Algorithmic bytes per edge: indices 4 B and species 4 B per atom, shifts
    12 B per non-first atom, float64 positions 24 B read and gradient 24 B added per atom, the
    parameter row; timed over `reps` evaluations."""
    import torch

    from kups_gb300 import bonded

    pos, system, n_per = _chains()
    S = int(system.max()) + 1
    species = (np.arange(len(pos)) % 2).astype(np.int32)
    tril = np.tile([40.0, 0, 40.0, 0, 0, 40.0], (S, 1))
    base = (np.arange(S) * n_per)[:, None]
    idx = lambda offs, lo, hi: (base + np.arange(lo, hi)[None, :])[..., None] + np.asarray(offs)
    T = 2
    terms = [
        bonded.BondedTerm(bonded.HarmonicBondParameters(("A", "B"), np.full((T, T), 1.5), np.full((T, T), 2.0)),
                          idx([0, 1], 0, n_per - 1).reshape(-1, 2)),
        bonded.BondedTerm(bonded.HarmonicAngleParameters(("A", "B"), np.full((T,) * 3, 109.5), np.full((T,) * 3, 0.01)),
                          idx([0, -1, 1], 1, n_per - 1).reshape(-1, 3)),
        bonded.BondedTerm(bonded.DihedralParameters(("A", "B"), np.full((T,) * 4, 0.1), np.full((T,) * 4, 3.0),
                                                    np.full((T,) * 4, np.pi)), idx([0, 1, 2, 3], 0, n_per - 3).reshape(-1, 4)),
        bonded.BondedTerm(bonded.InversionParameters(("A", "B"), np.zeros((T,) * 4), np.full((T,) * 4, 0.05)),
                          idx([0, -1, 1, 2], 1, n_per - 2).reshape(-1, 4)),
    ]
    bonded.evaluate(terms, pos, system, species, tril)  # warm-up, status checked
    from kups_gb300 import _lib
    from kups_gb300.neighborlist import new_status, read_status

    dev = "cuda"
    p = torch.as_tensor(pos, device=dev)
    sy = torch.as_tensor(system, device=dev, dtype=torch.int32)
    sp = torch.as_tensor(species, device=dev, dtype=torch.int32)
    tr = torch.as_tensor(tril, device=dev)
    energy = torch.zeros(S, dtype=torch.float64, device=dev)
    grad = torch.zeros_like(p)
    gtril = torch.zeros((S, 6), dtype=torch.float64, device=dev)
    status = new_status()

    def timed():
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            for t in terms:  # energies and gradients add up across terms and repetitions
                t.add_to(p, sy, sp, tr, energy, grad, gtril, status)
        e1.record()
        torch.cuda.synchronize()
        _lib.raise_status(read_status(status))
        return e0.elapsed_time(e1) / reps

    ms = timed()
    for t in terms:
        t.fp32 = True
    ms32 = timed()
    for t in terms:
        t.fp32 = False
    # MC energy change of one moved atom per chain (all systems in one call per term)
    rng = np.random.default_rng(4)
    ch = torch.as_tensor((np.arange(S) * n_per + rng.integers(0, n_per, S)).astype(np.int32), device=dev)
    newp = (p[ch.long()] + torch.as_tensor(rng.normal(scale=0.2, size=(S, 3)), device=dev)).contiguous()
    delta = torch.zeros(S, dtype=torch.float64, device=dev)
    dws = torch.empty(_lib.load().kups_bonded_delta_workspace_bytes(p.shape[0]), dtype=torch.uint8, device=dev)
    def delta_all():
        for t in terms:
            t.add_delta(p, sy, sp, tr, ch, newp, None, delta, dws, status)

    def timed_delta(run):
        run()
        torch.cuda.synchronize()
        d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d0.record()
        for _ in range(reps):
            run()
        d1.record()
        torch.cuda.synchronize()
        _lib.raise_status(read_status(status))
        return d0.elapsed_time(d1) / reps

    ms_delta_eager = timed_delta(delta_all)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        delta_all()  # warm-up on the capturing stream
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        delta_all()  # every launch of the four terms (memset, slot table, edge scan) in one graph
    ms_delta = timed_delta(graph.replay)
    for t in terms:
        t.fp32 = True
    delta_all()
    torch.cuda.synchronize()
    graph32 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph32):
        delta_all()
    ms_delta32 = timed_delta(graph32.replay)
    for t in terms:
        t.fp32 = False
    lib = _lib.load()
    n_edges = sum(t._edges.shape[0] for t in terms)
    nbytes = sum(t._edges.shape[0] * (t.order * (4 + 4 + 24 + 24) + 12 * (t.order - 1)
                                     + 8 * lib.kups_bonded_param_count(t.parameters.kind)) for t in terms)
    peak, kind = measured_peak()
    gbs, gbs32 = nbytes / (ms / 1e3) / 1e9, nbytes / (ms32 / 1e3) / 1e9
    return {"workload": f"{S} chains x {n_per} atoms: bonds, angles, dihedrals, inversions ({n_edges} edges)",
            "ms_per_evaluation": ms, "edges_per_s": n_edges / (ms / 1e3),
            "ms_per_evaluation_fp32": ms32, "edges_per_s_fp32": n_edges / (ms32 / 1e3),
            "mc_delta": {"ms_per_call": ms_delta, "ms_per_call_fp32": ms_delta32, "ms_per_call_eager": ms_delta_eager,
                         "moved_atoms": S,
                         "note": "one moved atom per chain, four terms, each moved atom's edges from the incidence "
                                 "lists; ms_per_call replays the four calls from a CUDA graph, eager is "
                                 "host-launched"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_source": kind, "note": "float64 atomics into the gradient, four launches per "
                                                      "evaluation, buffers allocated once"},
            "roofline_fp32": {"bound": "hbm", "achieved": gbs32, "peak": peak, "unit": "GB/s",
                              "frac": gbs32 / peak, "peak_source": kind,
                              "note": "per-edge arithmetic in float32, sums in float64"}}


def run_observables(a, reps=20):
    """kups_virial_stress with every output (atomic, molecular and lattice stress, kinetic energy,
    pressure) on 64 systems of 8000 three-atom molecules (1 536 000 atoms, positions wrapped atom
    by atom).  Algorithmic bytes per atom: positions, dU/dx and momenta 24 B each, mass 8 B,
    system and group 4 B each (88 B, each array read once); timed over `reps` calls with the
    buffers allocated once."""
    import torch

    from kups_gb300 import _lib
    from kups_gb300.neighborlist import _stream, new_status, read_status

    S, n_mol = 64, 8000
    rng = np.random.default_rng(9)
    tril = np.tile([45.0, 1.0, 44.0, -2.0, 0.5, 46.0], (S, 1))
    n = S * n_mol * 3
    sysi = np.repeat(np.arange(S), n_mol * 3)
    frac = np.repeat(rng.uniform(-0.5, 0.5, (S * n_mol, 3)), 3, axis=0) + rng.normal(scale=0.02, size=(n, 3))
    frac = (frac + 0.5) % 1.0 - 0.5
    L = np.zeros((S, 3, 3))
    L[:, [0, 1, 1, 2, 2, 2], [0, 0, 1, 0, 1, 2]] = tril
    dev = "cuda"
    t = lambda x, dt=torch.float64: torch.as_tensor(x, dtype=dt, device=dev).contiguous()
    pos, grad, mom = t(np.einsum("na,nab->nb", frac, L[sysi])), t(rng.normal(size=(n, 3))), t(rng.normal(size=(n, 3)))
    mass, sy, grp = t(rng.uniform(1, 16, n)), t(sysi, torch.int32), t(np.arange(n) // 3, torch.int32)
    tr, gt = t(tril), t(rng.normal(size=(S, 6)))
    outs = [torch.empty(S * 9, dtype=torch.float64, device=dev) for _ in range(3)]
    ke, pr = torch.empty(S, dtype=torch.float64, device=dev), torch.empty(S, dtype=torch.float64, device=dev)
    lib = _lib.load()
    G = S * n_mol
    wsb = lib.kups_virial_stress_workspace_bytes(S, G)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    status = new_status()

    def call():
        _lib.check(lib.kups_virial_stress(pos.data_ptr(), grad.data_ptr(), sy.data_ptr(), n, tr.data_ptr(),
                                          gt.data_ptr(), S, grp.data_ptr(), G, mom.data_ptr(), mass.data_ptr(),
                                          outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(),
                                          ke.data_ptr(), pr.data_ptr(), ws.data_ptr(), wsb, status.data_ptr(),
                                          _stream()), "kups_virial_stress")

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        call()
    e1.record()
    torch.cuda.synchronize()
    _lib.raise_status(read_status(status))
    ms = e0.elapsed_time(e1) / reps
    peak, kind = measured_peak()
    gbs = n * 88 / (ms / 1e3) / 1e9
    return {"workload": f"{S} systems x {n_mol} three-atom molecules ({n} atoms), all outputs", "ms_per_call": ms,
            "atoms_per_s": n / (ms / 1e3),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_source": kind, "note": "float64 throughout; molecular centres take three extra "
                                                      "passes (anchor, minimum-image sums, centre)"}}


def run_mliap(a, reps=10):
    """Local MLIAP energy and forces (the reference's test model: embedding 0.1, message
    h_j / (|d| + 1), linear readout) on 256 argon-like systems of 500 atoms at rc 5 A: graph by
    kups_neighborlist_build, model and gradients in torch."""
    import torch

    from kups_gb300 import mliap, workloads

    W = workloads.batched_uneven_lj(n_systems=256, n_min=500, n_max=500, seed=3)
    emb = torch.full((3, 4), 0.1, dtype=torch.float64, device="cuda")
    w = torch.full((4, 1), 0.1, dtype=torch.float64, device="cuda")
    pot = mliap.LocalMLIAP(lambda z: emb[z], lambda h1, h2, d: h2 / (d.norm(dim=-1, keepdim=True) + 1.0),
                           lambda h, m: ((h + m) @ w).squeeze(-1))
    pos = torch.as_tensor(W.positions, device="cuda")
    z = torch.zeros(W.n_atoms, dtype=torch.int64, device="cuda")
    sy = torch.as_tensor(W.system, device="cuda")
    tr = torch.as_tensor(W.tril, device="cuda")
    cut = np.full(W.n_systems, 5.0)
    pot.energy(pos, z, sy, tr, cut)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        res = pot.energy(pos, z, sy, tr, cut)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return {"workload": f"{W.n_systems} systems x 500 atoms, rc 5 A, reference test model", "ms_per_evaluation": ms,
            "atoms_per_s": W.n_atoms / (ms / 1e3), "note": "energy + dE/dx + dE/dtril; graph on the device, model in torch"}


def run_argon(a, torch):
    """Latency of the single-system argon NVT workload (864 atoms, fcc a = 5.74 A, rc 8.5 A +
    1 A skin, BAOAB dt 2 fs, 94.4 K): one persistent launch of 1000 steps on one CTA."""
    from kups_gb300 import md, workloads

    W = workloads.argon_fcc()
    prop = md.make_baoab_langevin_step()
    packed = md.pack(state_from_workload(W, torch))
    shape = None
    if not a.no_autotune:
        from kups_gb300.autotune import autotune_md

        shape = autotune_md(prop, packed, steps=100)
    prop.run_packed(packed, 20, seed=3, step0=0)
    torch.cuda.synchronize()
    steps = 1000
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    prop.launch(packed, steps, seed=3, step0=20, virial=False)
    t1.record()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    # the same system in float64 as the reference computes it: neighbour list rebuilt every step,
    # float64 LJ over the edges and float64 integrator blocks (kups_gb300.md.LennardJonesMD64)
    sim64 = md.LennardJonesMD64(state_from_workload(W, torch), "baoab", seed=3)
    sim64.run(20)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    sim64.run(steps)
    f1.record()
    torch.cuda.synchronize()
    sim64.check()
    ms64 = f0.elapsed_time(f1)
    return {"workload": "argon NVT: 864 atoms (6x6x6 fcc, a 5.74 A), rc 8.5 A + 1 A skin, BAOAB dt 2 fs, 94.4 K",
            "us_per_step": ms / steps * 1e3, "value": W.n_atoms * steps / (ms / 1e3), "unit": "atom-steps/s",
            "fp64": {"us_per_step": ms64 / steps * 1e3, "value": W.n_atoms * steps / (ms64 / 1e3),
                     "path": "float64 step by step: neighbour list every step (rc 8.5 A), float64 LJ over the "
                             "edges, float64 BAOAB blocks; 7 launches per step"},
            "launch_shape": {"block_threads": prop.block_threads or 1024, "min_lanes_per_atom": prop.min_lanes_per_atom or 2,
                             "chosen_by": "kups_gb300.autotune.autotune_md" if shape else "library default"}}


def _melt_sim(W, torch, real_space="auto", integrator="velocity_verlet", positions=None, temperature=None,
              friction=None):
    from kups_gb300 import ewald

    c = lambda x, dt=None: torch.as_tensor(np.asarray(x), dtype=dt).cuda()
    prm = ewald.EwaldParameters(torch.tensor([W.alpha]), torch.tensor([W.cutoff]), torch.as_tensor(W.kvec_n))
    pos = W.positions if positions is None else positions
    parts = ewald.EwaldParticles(c(pos), c(W.charges), c(np.zeros(len(W.charges), np.int32)), c(W.species))
    return ewald.LJEwaldMD(parts, c(W.masses), c(W.tril), prm, W.time_step, W.sigma, W.epsilon, [W.cutoff],
                           integrator=integrator, temperature=temperature, friction=friction, real_space=real_space)


def _against_float64(sim32, sim64, torch):
    """Energy and force error of the float32 all-pairs step against the float64 edge path at
    sim32's current positions (both add the same reciprocal and self terms)."""
    sim64.p.positions.copy_(sim32.p.positions)
    sim64._forces()
    torch.cuda.synchronize()
    g32, g64 = sim32.grad, sim64.grad
    rms = float(torch.sqrt(((g32 - g64) ** 2).mean() / (g64**2).mean()))
    e32, e64 = float(sim32.energy.item()), float(sim64.energy.item())
    return {"force_rms_rel": rms, "energy_rel": abs(e32 - e64) / abs(e64)}


def _nve_conservation(sim, steps, n_atoms, torch):
    """Total energy after every step of an NVE run, judged as the reference's NVE physics check
    does (ci/statistical/validate_nve_physics.py:29-62): slope of a linear fit per atom per step
    (bar 1e-8 eV) and std / |mean| (bar 5e-4)."""
    e = torch.empty(steps, dtype=torch.float64, device="cuda")
    for k in range(steps):
        sim.run(1)
        e[k] = sim.energy.sum() + sim.kinetic_energy().sum()
    sim.check()
    e = e.cpu().numpy()
    slope = float(np.polyfit(np.arange(steps), e, 1)[0])
    fluct = float(e.std() / abs(e.mean()))
    return {"steps": steps, "drift_ev_per_atom_step": abs(slope) / n_atoms, "relative_fluctuation": fluct,
            "drift_ok": abs(slope) / n_atoms < 1e-8, "fluctuation_ok": fluct < 5e-4, "mean_total_energy_ev": float(e.mean())}


def run_ewald_md(a):
    """LJ + Ewald NVE MD of the ionic melt: 2000 (+1 e) + 2000 (-1 e) ions in a 40 A cube,
    LB-mixed LJ (0.1 / 0.15 kcal/mol, 2.35 / 4.40 A), rc 12 A, alpha 0.3, |n| <= 8 k vectors
    in the reference's half-space layout, dt 1 fs, velocity Verlet; one step is captured
    once as a CUDA graph and replayed.  Device-timed over 1000 steps after 20.  Accuracy of the
    float32 all-pairs real space against the float64 edge path (kups_pair_edges, itself held to
    the float64 oracle at 1e-10) at the start and the end of the timed run; energy conservation
    of NVE runs from a melt equilibrated with BAOAB at 1200 K, with the float32 and with the
    float64 real space."""
    import torch

    from kups_gb300 import workloads

    W = workloads.ionic_melt()
    sim = _melt_sim(W, torch)
    ref = _melt_sim(W, torch, real_space="edges")
    sim.start(torch.as_tensor(W.momenta).cuda())
    ref.start(torch.as_tensor(W.momenta).cuda())
    from kups_gb300.autotune import autotune_lj_ewald

    tuned = autotune_lj_ewald(sim)  # untimed; before the step is captured
    acc0 = _against_float64(sim, ref, torch)
    sim.run(20)
    torch.cuda.synchronize()
    e0 = float((sim.energy + sim.kinetic_energy()).item())
    steps = 1000
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    sim.run(steps)
    t1.record()
    torch.cuda.synchronize()
    sim.check()
    ms = t0.elapsed_time(t1)
    e1 = float((sim.energy + sim.kinetic_energy()).item())
    acc1 = _against_float64(sim, ref, torch)
    n = len(W.charges)
    out = {"workload": f"ionic melt: {n} ions, 40 A cube, LJ + Ewald (alpha 0.3, rc 12 A, |n| <= 8), NVE dt 1 fs",
           "value": n * steps / (ms / 1e3), "unit": "atom-steps/s", "ms_per_step": ms / steps, "steps": steps,
           "relative_energy_change_from_start": (e1 - e0) / abs(e0),
           "real_space": ("all pairs (float hi/lo positions, per-warp hit queue), no list" if sim.allpairs
                          else "neighbour list every step"),
           "accuracy_vs_float64_path": {"start": acc0, "after_timed_run": acc1},
           "launch_shape": {"real_space_partner_shares": tuned.block_threads,
                            "chosen_by": "kups_gb300.autotune.autotune_lj_ewald",
                            "candidates_ms_per_force_evaluation": [[sp, ms] for sp, _, ms in tuned.table]},
           "fp32_roofline": ewald_fp32_roofline(W, n * steps / (ms / 1e3))}
    if getattr(a, "nve_check", True):
        from kups_gb300.units import FEMTO_SECOND

        eq = _melt_sim(W, torch, integrator="baoab", temperature=1200.0, friction=0.01 / FEMTO_SECOND)
        eq.start(torch.as_tensor(W.momenta).cuda())
        eq.run(2000)
        torch.cuda.synchronize()
        eq.check()
        pos_eq, mom_eq = eq.p.positions.cpu().numpy(), eq.mom.clone()
        cons = {}
        # 3000 steps for the float32 path: the slope of a 1000-step window varies between runs at
        # the 1e-8 level for both paths (a float64 run gave 1.0e-8 over 1000 steps)
        for tag, rs, nsteps in (("float32_all_pairs", "allpairs", 3000), ("float64_edges", "edges", 1000)):
            s2 = _melt_sim(W, torch, real_space=rs, positions=pos_eq)
            s2.start(mom_eq)
            cons[tag] = _nve_conservation(s2, nsteps, n, torch)
        out["nve_energy_conservation"] = {
            "start": "melt after 2000 BAOAB steps at 1200 K (friction 0.01 / fs) from the seeded lattice start",
            **cons}
    return out


def ewald_fp32_roofline(W, atom_steps_per_s):
    """FP32 work per atom-step of the LJ + Ewald step: half-list pairs within the cutoff x 70 flop
    (LJ 30 + erfc / exp 40) plus, per k vector, about 10 flop for the structure factor and 10 for
    the force (two complex products and the accumulation); peak derived from the SM count and
    the maximum SM clock (152 x 128 lanes x 2 flop x 2070 MHz on GB300)."""
    import torch

    n = len(W.charges)
    vol = abs(float(np.prod(np.asarray(W.tril).reshape(-1, 6)[0, [0, 2, 5]])))
    n_half = 4.0 / 3.0 * math.pi * W.cutoff**3 * n / vol / 2.0
    n_k = int(np.asarray(W.kvec_n).shape[1])
    flop = n_half * 70.0 + n_k * 20.0
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    peak = sms * 128 * 2 * 2070e6 / 1e12
    achieved = atom_steps_per_s * flop / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "flop_per_atom_step": flop, "peak_source": f"derived: {sms} SMs x 128 FP32 lanes x 2 flop x 2070 MHz"}


def run_gcmc(a):
    """Plain GCMC (uniform insertion, the reference's move set) against the learned insertion
    proposal on rigid CO2 in the 2000-atom porous host, replicated 2x2x1 (8000 atoms,
    50 x 50 x 25 A, 90/90/120 degrees), 0.1-10 bar log-spaced over the replicas, 298 K,
    Ewald alpha 0.25, 12 A cutoff.  Both production runs start from the same state; rates
    are device-timed (CUDA events around the persistent GCMC launches)."""
    from kups_gb300 import workloads
    from kups_gb300.mlp import learned_vs_plain

    setup = workloads.gcmc_co2_framework(n_replicas=a.gcmc_replicas)
    out = learned_vs_plain(setup, plain_steps=6000, snapshots=40, snapshot_every=100, train_steps=3000,
                           batch=16384, equil_steps=a.gcmc_equil, prod_steps=a.gcmc_prod, block=1000, temper=0.5)
    out["equilibration_steps"] = a.gcmc_equil
    out["production_steps"] = a.gcmc_prod
    out["roofline"] = gcmc_roofline(setup, out)
    out["workload"] = (f"GCMC rigid CO2 in a porous host: {a.gcmc_replicas} replicas, host 2000 atoms replicated "
                       "2x2x1 (8000), 0.1-10 bar, 298 K, Ewald alpha 0.25 rc 12 A, moves translate/rotate/"
                       "reinsert/insert/delete 1:1:1:1:1")
    out["unit"] = "accepted moves/s (all replicas)"
    out["note"] = ("production from a shared state that is not at equilibrium: CO2 condenses in the host channel "
                   "at 298 K and the loading keeps rising slowly under both samplers; loading agreement is tested "
                   "on a host that equilibrates (tests/test_gpu_gcmc.py)")
    out.pop("losses", None)
    return out


def gcmc_roofline(setup, out):
    """Per attempted move (one system-step), from the workload: n_cand = host + guest atoms within
    the cutoff of one moved atom (number density x 4/3 pi rc^3); B_alg = 16 B per candidate +
    n_k x (16 B S(k) read + 16 B write on accept + 8 B P(k)); F_alg = 6 moved positions (old and new
    of three atoms) x n_cand x 70 flop (LJ + erfc pair term) + 6 x n_k x 28 flop (phase and
    structure-factor update).  FP32 peak derived from the SM count and the maximum SM clock."""
    import torch

    t = np.asarray(setup.tril[0], float)
    vol = abs(t[0] * t[2] * t[5])
    apm = len(setup.motif_charges)
    n_guest = float(out["plain"]["loading_all"]) * apm
    rho = (float(setup.fw_count[0]) + n_guest) / vol
    rc = float(max(setup.rc_lj[0], setup.rc_ew[0]))
    n_cand = rho * 4.0 / 3.0 * math.pi * rc**3
    n_k = int(np.asarray(setup.kvec_n).shape[1])
    b_alg = 16.0 * n_cand + n_k * 40.0
    f_alg = 2 * apm * n_cand * 70.0 + 2 * apm * n_k * 28.0
    rate = float(out["plain"]["attempted_moves_per_s"])
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    peak32 = sms * 128 * 2 * 2070e6 / 1e12
    hbm, src = measured_peak()
    return {"bound": "fp32 issue", "unit": "TFLOP/s", "achieved": rate * f_alg / 1e12, "peak": peak32,
            "frac": rate * f_alg / 1e12 / peak32, "flop_per_move": f_alg, "bytes_per_move": b_alg,
            "hbm_achieved_gbs": rate * b_alg / 1e9, "hbm_peak_gbs": hbm, "hbm_frac": rate * b_alg / 1e9 / hbm,
            "hbm_peak_source": src, "candidates_per_moved_atom": n_cand, "n_kvecs": n_k,
            "peak_source": f"derived: {sms} SMs x 128 FP32 lanes x 2 flop x 2070 MHz"}


def state_from_workload(W, torch, device="cuda", pin=False):
    from kups_gb300 import md, potential

    def t(x, dt):
        v = torch.as_tensor(np.ascontiguousarray(x), dtype=dt)
        if device == "cpu":
            return v.pin_memory() if pin else v
        return v.to(device)

    prm = potential.LennardJonesParameters(("Ar",), torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(t(W.positions, torch.float64), t(W.momenta, torch.float64), t(W.masses, torch.float64),
                           t(W.species, torch.int32), t(W.system, torch.int32), None)
    systems = md.MDSystems(t(W.tril, torch.float64), t(W.time_step, torch.float64), t(W.temperature, torch.float64),
                           t(W.friction, torch.float64))
    return md.MDState(parts, systems, prm, skin=W.skin)


def run_e2e(a, W, torch):
    """Public propagator API driven from the host: ``FusedLennardJonesMD.propagate_host`` takes
    the dynamic state (positions, momenta, forces) in pinned host memory and updates it in
    place; each call copies it to the device, runs the steps and copies the new state back,
    and the next call starts from what came back, as a simulation loop on host buffers does;
    the per-system energies are read back after every call.  Inside, the batch runs as
    ``e2e_runs`` runs of whole systems whose copies overlap the other runs' launches.  The
    static arrays (species, system index, masses, cells and the per-system parameters) are
    uploaded once before the timed calls and passed as the same device tensors every call, so
    the propagator keeps its packed layouts and workspaces between calls: a system whose state
    came back unchanged resumes its Verlet list (kups_md_args.reuse_lists)."""
    from dataclasses import replace

    from kups_gb300 import md

    host = state_from_workload(W, torch, device="cpu", pin=True)
    n = W.n_atoms
    prop = md.make_baoab_langevin_step(steps_per_call=a.e2e_chunk)
    prop.block_threads, prop.min_lanes_per_atom = getattr(a, "tuned", (0, 0))
    hp = host.particles
    masses, species, system = (x.to("cuda") for x in (hp.masses, hp.species, hp.system))
    systems = md.MDSystems(*(x.to("cuda") for x in (host.systems.tril, host.systems.time_step,
                                                    host.systems.temperature, host.systems.friction_coefficient)))
    state = [md.MDState(md.MDParticles(hp.positions, hp.momenta, masses, species, system, None), systems,
                        host.lj_parameters, skin=host.skin)]
    energies = [None]

    def one_call(i):
        out = prop.propagate_host([i, 1], replace(state[0], step=i * a.e2e_chunk), chunks=a.e2e_runs)
        energies[0] = out.systems.potential_energy.cpu()
        state[0] = out

    one_call(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(a.e2e_calls):
        one_call(i + 1)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    steps = a.e2e_calls * a.e2e_chunk
    h2d = n * 3 * 8 * 3  # positions, momenta, forces (float64)
    d2h = n * 3 * 8 * 3 + W.n_systems * 8
    return {"value": n * steps / el, "unit": "atom-steps/s", "h2d_bytes_per_step": h2d / a.e2e_chunk,
            "d2h_bytes_per_step": d2h / a.e2e_chunk, "md_steps_per_call": a.e2e_chunk, "runs": a.e2e_runs,
            "api": "kups_gb300.md.FusedLennardJonesMD.propagate_host (dynamic state in pinned host memory, "
                   "updated in place, each call continuing from the state the previous call returned; runs "
                   "of whole systems with their copies overlapped; static topology and parameters uploaded "
                   "once)"}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    rate, cores, sample = cpu_baseline(a.systems, a.cpu_seconds, procs)
    line = {
        "impl": "reference",
        "metric": "batched LJ MD atom-steps/s",
        "value": rate,
        "unit": "atom-steps/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp64",
        "data": "synthetic (seeded)",
        "config": {"workload": "batched uneven LJ MD (sampled systems of the 4096-system batch)",
                   "implementation": "float64 NumPy restatement of the reference algorithm (reference JAX "
                                     "package not installable here: jax/jaxlib absent)"},
        "cpu_baseline": {"value": rate, "unit": "atom-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- profiling subcommands
# ``python bench.py --profile <what> [numbers...]`` runs one kernel's workload in the shape an ncu
# capture targets (the commands in profiles/*.md); nothing here is part of the JSON line.
MD_PHASES = ["setup+first build", "integrate", "list/ghosts", "forces", "kick+reduce", "write-back",
             "build:atoms", "build:ghosts", "thermostat/barostat", "build:list"]


def _events_ms(torch, fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def profile_md(n_sys=4096, equil=1000, steps=20, integrator="baoab"):
    """Fused MD on the batched workload: `equil` steps in four launches with the kernel's
    clock64 phase counters (ms/step, list builds per system, share of time per phase), then
    one launch of `steps` steps without counters (the launch `-s 4 -c 1` captures).
    integrator: baoab, velocity_verlet, csvr or csvr_npt (tau_T 100 fs, P0 1 bar, tau_P 1 ps,
    beta 2e-4 / bar)."""
    import torch

    from kups_gb300 import md
    from kups_gb300.units import FEMTO_SECOND

    n_sys, equil, steps = int(n_sys), int(equil), int(steps)
    W = workload(n_sys, 1)
    prop = md.FusedLennardJonesMD(integrator)
    state = state_from_workload(W, torch)
    if integrator in ("csvr", "csvr_npt"):
        bar = 6.241509074e-7  # eV / A^3
        full = lambda v: torch.full((n_sys,), float(v), dtype=torch.float64, device="cuda")
        state.systems.thermostat_time_constant = full(100 * FEMTO_SECOND)
        state.systems.target_pressure = full(bar)
        state.systems.pressure_coupling_time = full(1000 * FEMTO_SECOND)
        state.systems.compressibility = full(2e-4 / bar)
        state.systems.minimum_scale_factor = full(0.99)
    packed = md.pack(state)
    packed.rebuilds = torch.zeros(n_sys, device="cuda", dtype=torch.int32)
    packed.profile = torch.zeros(10, device="cuda", dtype=torch.int64)
    step0 = 0
    for chunk in [equil // 4] * 4:
        packed.rebuilds.zero_()
        packed.profile.zero_()
        ms = _events_ms(torch, lambda: prop.run_packed(packed, chunk, seed=1, step0=step0))
        step0 += chunk
        pr = packed.profile.cpu().double()
        pr /= pr[:6].sum() + pr[8]
        rb = packed.rebuilds.double()
        print(f"{chunk} steps: {ms / chunk:.3f} ms/step, list builds per system {rb.mean():.2f} "
              f"(max {rb.max():.0f}); " + " ".join(f"{n}={v:.3f}" for n, v in zip(MD_PHASES, pr.tolist())),
              flush=True)
    packed.profile = None
    ms = _events_ms(torch, lambda: prop.run_packed(packed, steps, seed=1, step0=step0))
    print(f"profiled launch: {steps} steps, {ms / steps:.3f} ms/step")


def profile_gcmc(replicas=1024, equil=3000, steps=40):
    """Plain GCMC of CO2 in the 2x2x1-replicated porous host: one launch of `equil` steps, then
    one launch of `steps` steps (the launch `-k regex:gcmc_kernel -s 1 -c 1` captures)."""
    import torch

    from kups_gb300 import gcmc as g
    from kups_gb300 import workloads

    replicas, equil, steps = int(replicas), int(equil), int(steps)
    mc = g.GCMC(workloads.gcmc_co2_framework(n_replicas=replicas), seed=1)
    mc.launch(equil)
    ms = _events_ms(torch, lambda: mc.launch(steps))
    mc.check()
    print(f"gcmc: {replicas} replicas, loading {mc.n_mol.float().mean().item():.2f}, {ms / steps * 1e3:.1f} us/step")
    # phase shares from the kernel's clock counters (a separate launch: the counters add barriers)
    mc.profile = torch.zeros(6, dtype=torch.int64, device="cuda")
    mc.launch(steps)
    mc.check()
    pr = mc.profile.cpu().double()
    names = ["proposal", "host atoms", "guests + moved molecule", "phase tables", "k sum", "acceptance + commit"]
    print("phases: " + " ".join(f"{n}={v / pr.sum():.3f}" for n, v in zip(names, pr.tolist())))
    mc.profile = None


def profile_mlp(train_steps=20, timed_train=200):
    """Learned-proposal network: `train_steps` training steps (batch 16384) on seeded points,
    then five 64^3 grid refreshes (forward of 262144 nodes, normaliser, CDF), five forward passes
    over 2^20 points alone and `timed_train` training steps, each timed with CUDA events."""
    import torch

    from kups_gb300.mlp import LearnedInsertionProposal

    net = LearnedInsertionProposal(seed=0, grid=64)
    gen = torch.Generator(device="cuda").manual_seed(0)
    data = torch.rand(200000, 3, dtype=torch.float64, device="cuda", generator=gen) * 0.3
    net.train(data, steps=int(train_steps), batch=16384)
    net.build_grid()
    pts = torch.rand(1 << 20, 3, dtype=torch.float64, device="cuda", generator=gen)
    net.forward(pts)
    torch.cuda.synchronize()
    flop_node = 2 * (64 * 256 + 2 * 256 * 256 + 256)
    ms = _events_ms(torch, lambda: [net.build_grid() for _ in range(5)]) / 5
    print(f"grid refresh: {ms:.3f} ms, {flop_node * 64**3 / ms / 1e9:.1f} TFLOP/s")
    ms = _events_ms(torch, lambda: [net.forward(pts) for _ in range(5)]) / 5
    print(f"forward of 2^20 points: {ms:.3f} ms, {flop_node * (1 << 20) / ms / 1e9:.1f} TFLOP/s")
    if int(timed_train) > 0:
        ms = _events_ms(torch, lambda: net.train(data, steps=int(timed_train), batch=16384)) / int(timed_train)
        print(f"train step (batch 16384): {ms:.3f} ms, {3 * flop_node * 16384 / ms / 1e9:.1f} TFLOP/s")


def profile_ewald(steps=50):
    """LJ + Ewald NVE of the ionic melt: 20 steps (graph capture and warm-up), then `steps`
    graph replays (the real-space launch `-k regex:real_packed_kernel -s 30 -c 1` captures)."""
    import torch

    from kups_gb300 import workloads

    W = workloads.ionic_melt()
    sim = _melt_sim(W, torch)
    sim.start(torch.as_tensor(W.momenta).cuda())
    sim.run(20)
    torch.cuda.synchronize()
    ms = _events_ms(torch, lambda: sim.run(int(steps)))
    sim.check()
    print(f"{steps} steps: {ms / int(steps):.4f} ms/step, {len(W.charges)} ions, {W.kvec_n.shape[1]} k vectors")


PROFILES = {"md": profile_md, "gcmc": profile_gcmc, "mlp": profile_mlp, "ewald": profile_ewald}


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--profile":
        what = sys.argv[2]
        PROFILES[what](*sys.argv[3:])
        return
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
