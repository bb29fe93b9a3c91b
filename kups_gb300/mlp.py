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

import torch

from . import _lib
from .neighborlist import _stream, new_status, read_status


def gemm(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None, bias=None, act: int = 0,
         alpha: float = 1.0, beta: float = 0.0, out2: torch.Tensor | None = None, gate=None, gate_kind: int = 0,
         status=None) -> torch.Tensor:
    """out = act(alpha * a @ b.T + beta * out + bias) (* gate'), tensors of any strides (2-D)."""
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
        float(beta), int(act), st.data_ptr(), _stream())
    _lib.check(rc, "kups_gemm_bf16")
    if status is None:
        _lib.raise_status(read_status(st))
    return out
