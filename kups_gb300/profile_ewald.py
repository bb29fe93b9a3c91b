"""Timing harness of the LJ + Ewald MD step on the ionic melt (4000 ions, 40 A cube,
rc 12 A, alpha 0.3, |n| <= 8 half-space k vectors, velocity Verlet dt 1 fs).

    python -m kups_gb300.profile_ewald [steps]

Builds the melt, runs 20 steps (graph capture and warm-up), then `steps` steps (default 50)
replayed from the captured CUDA graph, and prints ms per step.  An ncu capture of the
real-space kernel targets this command with -k regex:real_packed_kernel -s 30 -c 1.
"""

from __future__ import annotations

import sys

import numpy as np
import torch

from . import ewald, workloads


def main(argv):
    steps = int(argv[0]) if argv else 50
    W = workloads.ionic_melt()
    c = lambda x, dt=None: torch.as_tensor(np.asarray(x), dtype=dt).cuda()
    prm = ewald.EwaldParameters(torch.tensor([W.alpha]), torch.tensor([W.cutoff]), torch.as_tensor(W.kvec_n))
    parts = ewald.EwaldParticles(c(W.positions), c(W.charges), c(np.zeros(len(W.charges), np.int32)), c(W.species))
    sim = ewald.LJEwaldMD(parts, c(W.masses), c(W.tril), prm, W.time_step, W.sigma, W.epsilon, [W.cutoff])
    sim.start(c(W.momenta))
    sim.run(20)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.run(steps)
    e1.record()
    torch.cuda.synchronize()
    sim.check()
    print(f"{steps} steps: {e0.elapsed_time(e1) / steps:.4f} ms/step, {len(W.charges)} ions, "
          f"{W.kvec_n.shape[1]} k vectors", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
