"""Timing / profiling driver of the GCMC step and the learned-proposal network.

    python -m kups_gb300.profile_gcmc gcmc [replicas] [equilibration_steps] [profiled_steps]
    python -m kups_gb300.profile_gcmc mlp [train_steps]

``gcmc``: CO2 in the 2x2x1-replicated porous host, one equilibration launch then
one launch of ``profiled_steps`` plain GCMC steps (the launch an ncu capture
targets with ``-k regex:gcmc_kernel -s 1 -c 1``); prints device ms per step.
``mlp``: trains the proposal network ``train_steps`` steps (batch 16384) on
seeded points, then times the 64^3 grid refresh (forward of 262144 nodes,
normaliser and CDF) and 200 training steps with CUDA events.
"""

from __future__ import annotations

import sys

import torch


def _ms(fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def gcmc(replicas=1024, equil=3000, steps=40):
    from . import gcmc as g, workloads

    mc = g.GCMC(workloads.gcmc_co2_framework(n_replicas=replicas), seed=1)
    mc.launch(equil)
    ms = _ms(lambda: mc.launch(steps))
    mc.check()
    print(f"gcmc: {replicas} replicas, loading {mc.n_mol.float().mean().item():.2f}, "
          f"{ms / steps * 1e3:.1f} us/step")


def mlp(train_steps=20):
    from .mlp import LearnedInsertionProposal

    net = LearnedInsertionProposal(seed=0, grid=64)
    gen = torch.Generator(device="cuda").manual_seed(0)
    data = torch.rand(200000, 3, dtype=torch.float64, device="cuda", generator=gen) * 0.3
    net.train(data, steps=train_steps, batch=16384)
    net.build_grid()
    torch.cuda.synchronize()
    flop_node = 2 * (64 * 256 + 2 * 256 * 256 + 256)
    ms = _ms(lambda: [net.build_grid() for _ in range(5)]) / 5
    print(f"grid refresh: {ms:.3f} ms, {flop_node * 64**3 / ms / 1e9:.1f} TFLOP/s")
    ms = _ms(lambda: net.train(data, steps=200, batch=16384)) / 200
    print(f"train step (batch 16384): {ms:.3f} ms, {3 * flop_node * 16384 / ms / 1e9:.1f} TFLOP/s")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "gcmc"
    args = [int(x) for x in sys.argv[2:]]
    {"gcmc": gcmc, "mlp": mlp}[what](*args)
