"""Learned GCMC insertion proposal: a small MLP on tcgen05 tensor cores.

No counterpart exists in the reference; the proposal plugs into the
insertion move's log proposal ratio (the ``ChangesFn`` hook,
src/kups/mcmc/moves.py:92-98; summed into the acceptance at
src/kups/core/propagator.py:330-334).

Network: 64 Fourier features of the fractional position f (sin / cos of
2 pi m . f for 32 fixed integer vectors m) -> 3 hidden layers of width 256
(softplus) -> 1 output g(f), BF16 weights and activations, FP32
accumulation (``kups_gemm_bf16``).  The density is exp(g) evaluated on the
nodes of a periodic 64^3 grid and interpolated trilinearly; its exact
normaliser is the node mean, and sampling is exact (cell by its mass, then
a corner by its weight, then per-axis linear densities), so the proposal
density q(x) that enters the acceptance ratio is the one the sampler draws
from.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status
from .units import BOLTZMANN_CONSTANT, KILO_JOULE, MOL

EV_TO_KJ_PER_MOL = MOL / KILO_JOULE


def gemm(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None, bias=None, act: int = 0,
         alpha: float = 1.0, beta: float = 0.0, out2: torch.Tensor | None = None, gate=None, gate_kind: int = 0,
         split_k: int = 1, status=None) -> torch.Tensor:
    """out = act(alpha * a @ b.T + beta * out + bias) (* gate'), tensors of any strides (2-D).

    split_k > 1 adds alpha * a @ b.T into a float32 ``out`` (beta must be 1)."""
    m, k = a.shape
    n, k2 = b.shape
    if k != k2:
        raise ValueError("inner dimensions differ")
    if out is None:
        out = torch.empty((m, n), device="cuda", dtype=torch.float32)
    for t in (a, b, out) + ((out2,) if out2 is not None else ()):
        if t.dtype not in (torch.float32, torch.bfloat16) or not t.is_cuda:
            raise TypeError("operands must be float32 or bfloat16 CUDA tensors")
    st = status if status is not None else new_status()
    bf = lambda t: int(t.dtype == torch.bfloat16)
    g = gate if gate is not None else None
    rc = _lib.load().kups_gemm_bf16(
        a.data_ptr(), bf(a), a.stride(0), a.stride(1), b.data_ptr(), bf(b), b.stride(0), b.stride(1),
        out.data_ptr(), bf(out), out.stride(0), out.stride(1),
        out2.data_ptr() if out2 is not None else None, bf(out2) if out2 is not None else 0,
        out2.stride(0) if out2 is not None else 0, out2.stride(1) if out2 is not None else 0,
        bias.data_ptr() if bias is not None else None, g.data_ptr() if g is not None else None, int(gate_kind),
        g.stride(0) if g is not None else 0, g.stride(1) if g is not None else 0, m, n, k, float(alpha),
        float(beta), int(act), int(split_k), st.data_ptr(), _stream())
    _lib.check(rc, "kups_gemm_bf16")
    if status is None:
        _lib.raise_status(read_status(st))
    return out


N_PARAMS = 148481
OFFSETS = {"W1": (0, (256, 64)), "b1": (16384, (256,)), "W2": (16640, (256, 256)), "b2": (82176, (256,)),
           "W3": (82432, (256, 256)), "b3": (147968, (256,)), "w4": (148224, (256,)), "b4": (148480, (1,))}


def default_frequencies(seed: int = 7, max_order: int = 4) -> np.ndarray:
    """32 integer frequency vectors: the 13 of the half space of {-1, 0, 1}^3 \\ {0},
    then 19 distinct seeded draws from [-max_order, max_order]^3 (no sign-duplicates)."""
    out, seen = [], set()

    def add(m):
        m = tuple(int(v) for v in m)
        neg = tuple(-v for v in m)
        if m == (0, 0, 0) or m in seen or neg in seen:
            return
        seen.add(m)
        out.append(m)

    for m in np.stack(np.meshgrid(*[np.arange(-1, 2)] * 3, indexing="ij"), -1).reshape(-1, 3):
        add(m)
    rng = np.random.default_rng(seed)
    while len(out) < 32:
        add(rng.integers(-max_order, max_order + 1, 3))
    return np.array(out[:32], np.int32)


class LearnedInsertionProposal:
    """MLP log-density g(f) on fractional coordinates and its 64^3 grid sampler.

    Every step runs on the library's kernels: kups_mlp_nce_batch draws the
    batch, kups_mlp_bwd runs forward + backward on the tensor cores,
    kups_mlp_adam updates; kups_mlp_grid_norm evaluates the network on the grid
    nodes and builds the sampler's float64 CDF.
    """

    def __init__(self, seed: int = 0, freq: np.ndarray | None = None, grid: int = 64, floor: float = 0.05,
                 temper: float = 1.0):
        dev = "cuda"
        self.param = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.param_bf16 = torch.zeros(N_PARAMS, dtype=torch.bfloat16, device=dev)
        self.param_bf16_t = torch.zeros(2 * 256 * 256, dtype=torch.bfloat16, device=dev)
        self.grad = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.m = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.v = torch.zeros(N_PARAMS, dtype=torch.float32, device=dev)
        self.freq = torch.as_tensor(default_frequencies() if freq is None else np.asarray(freq, np.int32),
                                    device=dev).contiguous()
        self.net = _lib.Mlp(self.param.data_ptr(), self.param_bf16.data_ptr(), self.grad.data_ptr(),
                            self.m.data_ptr(), self.v.data_ptr(), self.freq.data_ptr(), self.param_bf16_t.data_ptr())
        self.grid, self.floor, self.temper = int(grid), float(floor), float(temper)
        self.node = torch.zeros(self.grid ** 3, dtype=torch.float32, device=dev)
        self.cdf = torch.zeros(self.grid ** 3 + 1, dtype=torch.float64, device=dev)
        self.status = new_status()
        self.t = 0
        self._ws = None
        _lib.check(_lib.load().kups_mlp_init(C.byref(self.net), int(seed) & (2**64 - 1), _stream()), "kups_mlp_init")

    def _workspace(self, n):
        nbytes = _lib.load().kups_mlp_workspace_bytes(int(n))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        return self._ws

    def params(self) -> dict:
        flat = self.param.cpu().numpy()
        return {k: flat[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFFSETS.items()}

    def forward(self, f: torch.Tensor) -> torch.Tensor:
        f = f.to(torch.float64).contiguous()
        g = torch.empty(f.shape[0], dtype=torch.float32, device="cuda")
        ws = self._workspace(f.shape[0])
        _lib.check(_lib.load().kups_mlp_fwd(C.byref(self.net), f.data_ptr(), f.shape[0], g.data_ptr(), ws.data_ptr(),
                                            ws.numel(), self.status.data_ptr(), _stream()), "kups_mlp_fwd")
        return g

    def backward(self, f: torch.Tensor, label: torch.Tensor, loss: torch.Tensor | None = None):
        """Adds dL/dparam of the batch to ``self.grad`` (and L to ``loss``)."""
        f = f.to(torch.float64).contiguous()
        label = label.to(torch.float32).contiguous()
        ws = self._workspace(f.shape[0])
        _lib.check(_lib.load().kups_mlp_bwd(C.byref(self.net), f.data_ptr(), label.data_ptr(), f.shape[0],
                                            loss.data_ptr() if loss is not None else None, ws.data_ptr(), ws.numel(),
                                            self.status.data_ptr(), _stream()), "kups_mlp_bwd")

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.t += 1
        _lib.check(_lib.load().kups_mlp_adam(C.byref(self.net), self.t, lr, beta1, beta2, eps, _stream()),
                   "kups_mlp_adam")

    def train(self, data: torch.Tensor, steps: int, batch: int = 16384, lr: float = 2e-3, seed: int = 1,
              lr_final: float | None = None, log_every: int = 0):
        """Noise-contrastive training on fractional positions ``data`` [N, 3]; returns sampled losses."""
        lib = _lib.load()
        data = data.to(torch.float64).contiguous()
        x = torch.empty((batch, 3), dtype=torch.float64, device="cuda")
        y = torch.empty(batch, dtype=torch.float32, device="cuda")
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        losses = []
        lr_final = lr if lr_final is None else lr_final
        for it in range(steps):
            _lib.check(lib.kups_mlp_nce_batch(data.data_ptr(), data.shape[0], batch, int(seed), it, x.data_ptr(),
                                              y.data_ptr(), _stream()), "kups_mlp_nce_batch")
            log = log_every and (it % log_every == 0 or it == steps - 1)
            if log:
                loss.zero_()
            self.backward(x, y, loss if log else None)
            frac = it / max(1, steps - 1)
            self.adam(lr * (lr_final / lr) ** frac)
            if log:
                losses.append((it, float(loss.item())))
        self.check()
        return losses

    def build_grid(self):
        """Node values and CDF of the sampler from the current network."""
        n = self.grid ** 3
        ws = self._workspace(n)
        _lib.check(_lib.load().kups_mlp_grid_norm(C.byref(self.net), self.grid, self.temper, self.floor,
                                                  self.node.data_ptr(),
                                                  self.cdf.data_ptr(), ws.data_ptr(), ws.numel(),
                                                  self.status.data_ptr(), _stream()), "kups_mlp_grid_norm")
        self.check()
        return self.node, self.cdf

    def sample(self, n: int, seed: int = 0):
        f = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        lq = torch.empty(n, dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().kups_proposal_sample(self.node.data_ptr(), self.cdf.data_ptr(), self.grid, n, seed,
                                                    f.data_ptr(), lq.data_ptr(), _stream()), "kups_proposal_sample")
        return f, lq

    def log_density(self, f: torch.Tensor) -> torch.Tensor:
        f = f.to(torch.float64).contiguous()
        lq = torch.empty(f.shape[0], dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().kups_proposal_log_density(self.node.data_ptr(), self.cdf.data_ptr(), self.grid,
                                                         f.data_ptr(), f.shape[0], lq.data_ptr(), _stream()),
                   "kups_proposal_log_density")
        return lq

    def check(self):
        _lib.raise_status(read_status(self.status))


def _timed_run(mc, steps, block):
    """Runs ``steps`` MC steps in launches of ``block`` steps; returns device ms (the whole
    sequence), accepted/attempted per move kind and the kernel's per-block sums of U, N, U N,
    N^2, U^2 of every system [blocks, S, 5] (every step counted, one read-back at the end)."""
    att0, acc0 = mc.attempted.clone(), mc.accepted.clone()
    nb = steps // block
    sums = torch.empty((nb,) + tuple(mc.obs.shape), dtype=torch.float64, device=mc.obs.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for b in range(nb):
        mc.obs.zero_()
        mc.launch(block)
        sums[b].copy_(mc.obs)
    e1.record()
    torch.cuda.synchronize()
    mc.check()
    att = (mc.attempted - att0).sum(0).cpu().numpy()
    acc = (mc.accepted - acc0).sum(0).cpu().numpy()
    return e0.elapsed_time(e1), att, acc, sums.cpu().numpy()


def learned_vs_plain(setup, plain_steps=6000, snapshots=40, snapshot_every=100, train_steps=3000, batch=16384,
                     equil_steps=10000, prod_steps=5000, block=500, temper=0.5, floor=0.05, grid=64, seed=0,
                     groups=8, tune=True):
    """Plain GCMC from empty, centres of the molecules it holds as training data, NCE training,
    equilibration with the learned proposal, then plain and learned production runs from copies
    of that state.  Returns rates (accepted insertions / moves per second, device time) and the
    loading of each pressure group (replicas in order, ``groups`` equal groups) with its
    block-averaged standard error."""
    from . import gcmc

    mc = gcmc.GCMC(setup, seed=seed + 1)
    mc.launch(plain_steps)
    cent = []
    for _ in range(snapshots):
        mc.launch(snapshot_every)
        cent.append(mc.molecule_centres_frac())
    mc.check()
    data = torch.cat(cent)
    net = LearnedInsertionProposal(seed=seed, grid=grid, floor=floor, temper=temper)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    losses = net.train(data, steps=train_steps, batch=batch, lr=2e-3, lr_final=2e-4, seed=seed + 2,
                       log_every=max(1, train_steps // 4))
    net.build_grid()
    e1.record()
    torch.cuda.synchronize()
    train_ms = e0.elapsed_time(e1)
    mc.use_proposal(net)
    mc.launch(equil_steps)
    mc.check()
    out = {"training_positions": int(data.shape[0]), "train_ms": train_ms, "losses": losses,
           "replicas": setup.n_systems}
    S = setup.n_systems
    for tag, proposal in (("plain", None), ("learned", net)):
        run = mc.clone(seed=seed + 3)
        run.use_proposal(proposal)
        shape = None
        if tune:
            from .autotune import autotune_gcmc

            shape = autotune_gcmc(run)  # on clones of `run`'s state: `run` does not advance
        ms, att, acc, sums = _timed_run(run, prod_steps, block)
        m = sums / block  # block means of U, N, U N, N^2, U^2 per system
        loads = m[..., 1]
        g = loads.reshape(len(loads), groups, S // groups).mean(2)  # [blocks, groups]
        # heat of adsorption per block and pressure group, cov(U, N) / var(N) - kT with the
        # within-block covariances pooled over the group's replicas (a single replica's N can
        # stay constant for a whole block in the condensed channel)
        cov = (m[..., 2] - m[..., 0] * m[..., 1]).reshape(len(m), groups, S // groups).mean(2)
        var = (m[..., 3] - m[..., 1] ** 2).reshape(len(m), groups, S // groups).mean(2)
        kt = np.asarray(setup.temperature, np.float64).reshape(groups, S // groups).mean(1) * BOLTZMANN_CONSTANT
        with np.errstate(invalid="ignore", divide="ignore"):
            qg = (cov / var - kt[None, :]) * EV_TO_KJ_PER_MOL
        # a block whose N never changed in any of the group's replicas defines no heat of
        # adsorption: averaged over the blocks that do; null where fewer than two do
        q_ok = np.isfinite(qg) & (var > 0)
        q_n = q_ok.sum(0)
        q_mean = [float(qg[q_ok[:, j], j].mean()) if q_n[j] >= 2 else None for j in range(groups)]
        q_se = [float(qg[q_ok[:, j], j].std(ddof=1) / np.sqrt(q_n[j])) if q_n[j] >= 2 else None
                for j in range(groups)]
        out[tag] = {
            "ms_per_step": ms / prod_steps,
            "accepted_insertions_per_s": float(acc[3] / ms * 1e3),
            "accepted_moves_per_s": float(acc.sum() / ms * 1e3),
            "attempted_moves_per_s": float(att.sum() / ms * 1e3),
            "insert_acceptance": float(acc[3] / max(att[3], 1)),
            "delete_acceptance": float(acc[4] / max(att[4], 1)),
            "loading": g.mean(0).tolist(),
            "loading_se": (g.std(0, ddof=1) / np.sqrt(len(g))).tolist(),
            "loading_all": float(loads.mean()),
            "loading_all_se": float(loads.mean(1).std(ddof=1) / np.sqrt(len(loads))),
            "heat_of_adsorption_kj_mol": q_mean,
            "heat_of_adsorption_se": q_se,
            "heat_of_adsorption_blocks": q_n.tolist(),
            "launch_shape": ({"block_threads": shape.block_threads, "chosen_by": "kups_gb300.autotune.autotune_gcmc",
                              "candidates_ms_per_step": [[t, m] for t, _, m in shape.table]}
                             if shape is not None else {"block_threads": 128, "chosen_by": "library default"}),
        }
    lp, ll = np.array(out["plain"]["loading"]), np.array(out["learned"]["loading"])
    sp, sl = np.array(out["plain"]["loading_se"]), np.array(out["learned"]["loading_se"])
    out["loading_z"] = ((ll - lp) / np.sqrt(sp**2 + sl**2)).tolist()
    out["loading_all_z"] = (out["learned"]["loading_all"] - out["plain"]["loading_all"]) / np.sqrt(
        out["learned"]["loading_all_se"] ** 2 + out["plain"]["loading_all_se"] ** 2)
    out["insertion_gain"] = out["learned"]["accepted_insertions_per_s"] / max(out["plain"]["accepted_insertions_per_s"], 1e-30)
    return out
