"""Phase profile of the fused LJ MD kernel on the batched uneven LJ workload.

    python -m kups_gb300.profile_md [n_systems] [equilibration_steps] [profiled_steps] [integrator]

Packs the seeded workload, runs the equilibration in four launches (printing
ms/step, Verlet-list builds per system and the share of kernel time per
phase from the kernel's clock64 counters), then one launch of
`profiled_steps` steps (the launch an ncu capture targets with -s 4 -c 1).
`integrator` is baoab (default), verlet, csvr or csvr_npt (tau_T 100 fs, P0 1 bar,
tau_P 1 ps, beta 2e-4 / bar).
"""

from __future__ import annotations

import sys

import torch

from . import md, workloads

PHASES = ["setup+first build", "integrate", "list/ghosts", "forces", "kick+reduce", "write-back",
          "build:atoms", "build:ghosts", "thermostat/barostat", "build:list"]


def state_from_workload(W) -> md.MDState:
    from . import potential

    c = lambda x, dt: torch.as_tensor(x, dtype=dt).cuda()
    prm = potential.LennardJonesParameters(("Ar",), torch.as_tensor(W.sigma), torch.as_tensor(W.epsilon),
                                           torch.tensor([W.cutoff], dtype=torch.float64))
    parts = md.MDParticles(c(W.positions, torch.float64), c(W.momenta, torch.float64), c(W.masses, torch.float64),
                           c(W.species, torch.int32), c(W.system, torch.int32))
    systems = md.MDSystems(c(W.tril, torch.float64), c(W.time_step, torch.float64), c(W.temperature, torch.float64),
                           c(W.friction, torch.float64))
    return md.MDState(parts, systems, prm, skin=W.skin)


def main(argv):
    n_sys = int(argv[0]) if len(argv) > 0 else 4096
    equil = int(argv[1]) if len(argv) > 1 else 1000
    steps = int(argv[2]) if len(argv) > 2 else 20
    integrator = argv[3] if len(argv) > 3 else "baoab"
    W = workloads.batched_uneven_lj(n_systems=n_sys, seed=1)
    prop = md.FusedLennardJonesMD(integrator)
    state = state_from_workload(W)
    if integrator in ("csvr", "csvr_npt"):
        from .units import FEMTO_SECOND

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
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        prop.run_packed(packed, chunk, seed=1, step0=step0)
        e1.record()
        torch.cuda.synchronize()
        step0 += chunk
        pr = packed.profile.cpu().double()
        pr /= pr[:6].sum() + pr[8]
        rb = packed.rebuilds.double()
        print(f"{chunk} steps: {e0.elapsed_time(e1) / chunk:.3f} ms/step, list builds per system "
              f"{rb.mean():.2f} (max {rb.max():.0f}); " +
              " ".join(f"{n}={v:.3f}" for n, v in zip(PHASES, pr.tolist())), flush=True)
    packed.profile = None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    prop.run_packed(packed, steps, seed=1, step0=step0)
    e1.record()
    torch.cuda.synchronize()
    print(f"profiled launch: {steps} steps, {e0.elapsed_time(e1) / steps:.3f} ms/step")


if __name__ == "__main__":
    main(sys.argv[1:])
