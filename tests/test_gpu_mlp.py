"""tcgen05 BF16 GEMM against a float32 torch reference of the same (bf16-rounded) operands.

Bar: relative Frobenius error 1e-5 (exact bf16 products, float32 accumulation
in a different order).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def ref(a, b):
    return a.bfloat16().float() @ b.bfloat16().float().T


def rel(x, y):
    return float((x - y).norm() / y.norm().clamp_min(1e-30))


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (256, 256, 64), (384, 256, 256), (200, 100, 80), (128, 16, 16)])
def test_gemm_shapes(m, n, k):
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    a = torch.randn(m, k, device="cuda", generator=g)
    b = torch.randn(n, k, device="cuda", generator=g)
    c = gemm(a, b)
    assert rel(c, ref(a, b)) < 1e-5


def test_gemm_transposed_operands_bias_act_and_second_output():
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(3)
    a_t = torch.randn(96, 256, device="cuda", generator=g)  # a = a_t.T, shape 256 x 96
    b = torch.randn(64, 96, device="cuda", generator=g).bfloat16()
    bias = torch.randn(64, device="cuda", generator=g)
    out = torch.empty(256, 64, device="cuda")
    out2 = torch.empty(64, 256, device="cuda", dtype=torch.bfloat16)
    gemm(a_t.T, b, out, bias=bias, act=1, out2=out2.T)
    r = torch.relu(ref(a_t.T, b.float()) + bias)
    assert rel(out, r) < 1e-5
    assert rel(out2.float().T, r) < 1e-2


def test_gemm_accumulate_and_gate():
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(4)
    a = torch.randn(256, 128, device="cuda", generator=g)
    b = torch.randn(128, 128, device="cuda", generator=g)
    c0 = torch.randn(256, 128, device="cuda", generator=g)
    pre = torch.randn(256, 128, device="cuda", generator=g)
    c = c0.clone()
    gemm(a, b, c, alpha=0.5, beta=2.0, gate=pre, gate_kind=2)
    r = (0.5 * ref(a, b) + 2.0 * c0) * torch.sigmoid(pre)
    assert rel(c, r) < 1e-5
