"""Launch-shape autotuners: the fused Lennard-Jones MD kernel, the GCMC kernel and the
all-pairs LJ + Ewald real space.

The fused kernel's throughput depends on two launch choices that no formula fixes well
across workloads: threads per CTA (one CTA per SM owns one system at a time; more threads
hide more shared-memory latency but lengthen the barrier tails of small systems) and the
minimum number of lanes that share one atom's Verlet list in the force phase (more lanes
give finer work units at the end of a phase, fewer lanes fewer shuffle reductions).
``autotune_md`` times every candidate on a copy of the caller's packed state (the state is
restored after each trial, so tuning does not advance the simulation), keeps the fastest,
and caches it per workload signature (system count, largest system, densest system, cutoff
and skin, integrator), in memory and optionally in a JSON file.  Results of the tuned and
untuned kernels are the same up to float32 summation order.
"""

from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass

import torch

from . import _lib
from .neighborlist import read_status

BLOCK_THREADS = (512, 640, 768, 896, 1024)
MIN_LANES = (1, 2, 4)

_CACHE: dict[str, dict] = {}


@dataclass
class TunedShape:
    block_threads: int
    min_lanes_per_atom: int
    ms_per_step: float
    table: list  # [(block_threads, min_lanes, ms_per_step)] of every candidate


def signature(packed, prop) -> str:
    counts = (packed.sys_offset[1:] - packed.sys_offset[:-1]).to(torch.float64)
    return json.dumps({
        "systems": int(packed.n_systems), "max_atoms": int(packed.max_atoms),
        "density": round(float(packed.max_density), 4), "mean_atoms": round(float(counts.mean()), 1),
        "cutoff": round(float(packed.cutoff.max()), 3), "skin": round(float(packed.skin.max()), 3),
        "integrator": prop.integrator,
    }, sort_keys=True)


def _time(prop, packed, steps, seed):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    st = prop.launch(packed, steps, seed=seed, step0=0, virial=False)
    e1.record()
    torch.cuda.synchronize()
    status = read_status(st)
    return e0.elapsed_time(e1) / steps, status


def autotune_md(prop, packed, steps: int = 40, cache_file: str | None = None,
                block_threads=BLOCK_THREADS, min_lanes=MIN_LANES) -> TunedShape:
    """Time each (block_threads, min_lanes_per_atom) candidate for `steps` steps after one
    untimed launch of the same length (list builds and caches warm), set the fastest on
    `prop` and return it.  `packed` is left as it was."""
    key = signature(packed, prop)
    if key not in _CACHE and cache_file and os.path.exists(cache_file):
        with open(cache_file) as f:
            _CACHE.update(json.load(f))
    if key in _CACHE:
        c = _CACHE[key]
        prop.block_threads, prop.min_lanes_per_atom = c["block_threads"], c["min_lanes_per_atom"]
        return TunedShape(c["block_threads"], c["min_lanes_per_atom"], c["ms_per_step"], c["table"])
    backup = packed.clone_dynamic()
    valid0 = packed.forces_valid
    saved = (prop.block_threads, prop.min_lanes_per_atom)
    table = []
    best = (math.inf, None)
    for bt in block_threads:
        for ml in min_lanes:
            prop.block_threads, prop.min_lanes_per_atom = bt, ml
            _, st0 = _time(prop, packed, steps, seed=1)
            ms, st1 = _time(prop, packed, steps, seed=2)
            packed.restore_dynamic(backup)
            packed.forces_valid = valid0
            if st0.code != _lib.KUPS_OK or st1.code != _lib.KUPS_OK:
                table.append((bt, ml, None))
                continue
            table.append((bt, ml, ms))
            if ms < best[0]:
                best = (ms, (bt, ml))
    if best[1] is None:
        prop.block_threads, prop.min_lanes_per_atom = saved
        raise _lib.KupsError("no launch shape ran without a device error")
    prop.block_threads, prop.min_lanes_per_atom = best[1]
    _CACHE[key] = {"block_threads": best[1][0], "min_lanes_per_atom": best[1][1], "ms_per_step": best[0],
                   "table": table}
    if cache_file:
        with open(cache_file, "w") as f:
            json.dump(_CACHE, f, indent=1)
    return TunedShape(best[1][0], best[1][1], best[0], table)


GCMC_THREADS = (64, 128, 256)


def autotune_gcmc(mc, steps: int = 200, candidates=GCMC_THREADS) -> TunedShape:
    """Threads per system's CTA of the GCMC kernel (64, 128 or 256: more threads share a
    system's host-atom and k-vector loops, fewer fit more systems per SM), each timed for
    `steps` steps on a clone of the sampler's state (``GCMC.clone``: `mc` itself does not
    advance), after one untimed launch of the same length; the fastest is set on `mc` and
    cached per workload signature (systems, host atoms, k vectors, molecules, proposal)."""
    st = mc.setup
    key = json.dumps({"kernel": "gcmc", "systems": int(st.n_systems), "host_atoms": int(max(st.fw_count)),
                      "kvecs": int(st.kvec_n.shape[1]), "max_mol": int(st.max_mol),
                      "loading": round(float(mc.n_mol.float().mean()), 0), "learned": mc.proposal is not None},
                     sort_keys=True)
    if key in _CACHE:
        c = _CACHE[key]
        mc.block_threads = c["block_threads"]
        return TunedShape(c["block_threads"], 0, c["ms_per_step"], c["table"])
    table, best = [], (math.inf, None)
    for t in candidates:
        trial = mc.clone(seed=mc.seed)
        trial.block_threads = t
        trial.launch(steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        trial.launch(steps)
        e1.record()
        torch.cuda.synchronize()
        status = read_status(trial.status)
        ms = e0.elapsed_time(e1) / steps
        del trial
        if status.code != _lib.KUPS_OK:
            table.append((t, 0, None))
            continue
        table.append((t, 0, ms))
        if ms < best[0]:
            best = (ms, t)
    if best[1] is None:
        raise _lib.KupsError("no GCMC launch shape ran without a device error")
    mc.block_threads = best[1]
    _CACHE[key] = {"block_threads": best[1], "min_lanes_per_atom": 0, "ms_per_step": best[0], "table": table}
    return TunedShape(best[1], 0, best[0], table)


LJ_EWALD_SPLITS = (1, 2, 3, 4)


def autotune_lj_ewald(sim, calls: int = 30, candidates=LJ_EWALD_SPLITS) -> TunedShape:
    """Partner shares per 16-atom block of the all-pairs LJ + Ewald real space
    (``kups_lj_ewald_real_forces_packed``, terms bits 8-11; 0 is the library default, one share)
    for an ``ewald.LJEwaldMD`` whose real space runs without a list.
    Each candidate is timed over `calls` force evaluations at the current positions (a force
    evaluation does not advance the state), after one untimed call; the fastest is set on `sim`
    (before its step is captured as a CUDA graph) and cached per workload signature (systems,
    largest system, cutoffs).  The returned table lists (shares, 0, ms per force evaluation)."""
    if not sim.allpairs:
        return TunedShape(0, 0, math.nan, [])
    key = json.dumps({"kernel": "lj_ewald_real_packed", "systems": int(sim.s), "max_atoms": int(sim.max_atoms),
                      "rc": round(float(sim.rc_ew.max()), 3), "kvecs": int(sim.kn.shape[1])}, sort_keys=True)
    if key in _CACHE:
        c = _CACHE[key]
        sim.real_splits = c["block_threads"]
        return TunedShape(c["block_threads"], 0, c["ms_per_step"], c["table"])
    keep = sim.real_splits
    # two rounds over the candidates, the faster of each candidate's two timings kept: the first
    # calls of a process also pay one-time costs (module loading, first touches of memory)
    timed: dict = {}
    for _ in range(2):
        for sp in candidates:
            sim.real_splits = sp
            sim._forces()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(calls):
                sim._forces()
            e1.record()
            torch.cuda.synchronize()
            ok = read_status(sim.status).code == _lib.KUPS_OK
            ms = e0.elapsed_time(e1) / calls if ok else None
            prev = timed.get(sp, math.inf)
            timed[sp] = None if (ms is None or prev is None) else min(prev, ms)
    table, best = [], (math.inf, None)
    for sp in candidates:
        ms = timed[sp]
        table.append((sp, 0, ms))
        if ms is not None and ms < best[0]:
            best = (ms, sp)
    sim.real_splits = keep if best[1] is None else best[1]
    sim._forces()  # energy and gradient of the current state with the chosen shape
    torch.cuda.synchronize()
    if best[1] is None:
        raise _lib.KupsError("no LJ + Ewald launch shape ran without a device error")
    _CACHE[key] = {"block_threads": best[1], "min_lanes_per_atom": 0, "ms_per_step": best[0], "table": table}
    return TunedShape(best[1], 0, best[0], table)
