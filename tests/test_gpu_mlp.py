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


def test_gemm_split_k_and_softplus_output_gate():
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(5)
    a_t = torch.randn(3000, 256, device="cuda", generator=g)  # K = 3000 along rows
    b_t = torch.randn(3000, 64, device="cuda", generator=g).bfloat16()
    c = torch.zeros(256, 64, device="cuda")
    gemm(a_t.T, b_t.T, c, beta=1.0, split_k=12)
    assert rel(c, ref(a_t.T, b_t.T.float())) < 1e-5
    h = torch.nn.functional.softplus(torch.randn(256, 128, device="cuda", generator=g))
    a = torch.randn(256, 96, device="cuda", generator=g)
    b = torch.randn(128, 96, device="cuda", generator=g)
    out = torch.empty(256, 128, device="cuda")
    gemm(a, b, out, gate=h, gate_kind=3)
    assert rel(out, ref(a, b) * -torch.expm1(-h)) < 1e-5


# ----------------------------------------------------------------------------- learned proposal network
# Bars: forward g within relative 1e-4 (Frobenius) of the float64 oracle that
# rounds the same operands to bfloat16; gradients within relative 2e-3 per
# parameter block (isolated bfloat16 rounding flips of float32-vs-float64
# activations); Adam within 1e-6 absolute.


def _net(seed=3):
    from kups_gb300.mlp import LearnedInsertionProposal

    return LearnedInsertionProposal(seed=seed, grid=16)


def test_mlp_forward_matches_oracle():
    from oracle import mlp as om

    net = _net()
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 1, (3000, 3))
    g = net.forward(torch.as_tensor(x, device="cuda")).cpu().numpy()
    ref_g = om.forward(net.params(), x, net.freq.cpu().numpy())["g"]
    assert np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g) < 1e-4


def test_mlp_forward_many_tiles_per_cta_matches_oracle():
    """Ragged point count spanning two to three 256-point tiles per CTA (the weight-chunk ring
    runs across tile boundaries), against the oracle and against the layered training path."""
    from oracle import mlp as om

    net = _net(8)
    rng = np.random.default_rng(9)
    n = 152 * 256 * 2 + 77
    x = rng.uniform(-1, 2, (n, 3))  # any periodic image
    g = net.forward(torch.as_tensor(x, device="cuda")).cpu().numpy()
    ref_g = om.forward(net.params(), x, net.freq.cpu().numpy())["g"]
    assert np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g) < 1e-4
    assert np.isfinite(g).all()


def test_mlp_backward_matches_oracle():
    from oracle import mlp as om

    net = _net(4)
    rng = np.random.default_rng(1)
    n = 4096
    x = rng.uniform(0, 1, (n, 3))
    x[: n // 2] = 0.3 + 0.05 * rng.normal(size=(n // 2, 3))  # a data blob against uniform points
    y = (np.arange(n) < n // 2).astype(np.float32)
    loss = torch.zeros(1, device="cuda")
    net.backward(torch.as_tensor(x, device="cuda"), torch.as_tensor(y, device="cuda"), loss)
    grad = om.unflatten(net.grad.cpu().numpy())
    ref_loss, ref = om.loss_and_grad(net.params(), x, y, net.freq.cpu().numpy())
    assert abs(loss.item() - ref_loss) < 1e-5 * max(1.0, ref_loss)
    for k in ref:
        err = np.linalg.norm(grad[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-30)
        assert err < 2e-3, (k, err)


def test_mlp_adam_matches_oracle():
    from oracle import mlp as om

    net = _net(5)
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 1, (2048, 3))
    y = (rng.uniform(size=2048) < 0.5).astype(np.float32)
    p0 = net.param.cpu().numpy().astype(np.float64)
    net.backward(torch.as_tensor(x, device="cuda"), torch.as_tensor(y, device="cuda"))
    g = net.grad.cpu().numpy().astype(np.float64)
    net.adam(1e-3)
    p_ref, _, _ = om.adam(p0, g, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
    np.testing.assert_allclose(net.param.cpu().numpy(), p_ref, atol=1e-6)
    assert float(net.grad.abs().max()) == 0.0
    np.testing.assert_array_equal(net.param_bf16.float().cpu().numpy(), om.bf16(net.param.cpu().numpy()))


def test_grid_norm_matches_network_on_nodes():
    from oracle import mlp as om

    net = _net(6)
    node, cdf = net.build_grid()
    G = net.grid
    g = net.forward(torch.as_tensor(om.grid_nodes(G), device="cuda")).cpu().numpy()
    ref_node = om.grid_density(g, net.floor)
    np.testing.assert_allclose(node.cpu().numpy(), ref_node, rtol=2e-6)
    np.testing.assert_allclose(cdf.cpu().numpy(), om.cdf_from_node(node.cpu().numpy(), G), rtol=1e-12, atol=1e-12)


def _blob_data(n, rng, centres=((0.2, 0.3, 0.4), (0.7, 0.75, 0.1)), width=0.06):
    c = np.asarray(centres)[rng.integers(0, len(centres), n)]
    return (c + width * rng.normal(size=(n, 3))) % 1.0


def test_sampler_is_exact_for_its_density():
    from oracle import mlp as om

    net = _net(7)
    rng = np.random.default_rng(3)
    net.train(torch.as_tensor(_blob_data(50000, rng), device="cuda"), steps=60, batch=4096, lr=3e-3)
    net.grid = 4  # a coarse grid so every sub-cell bin is well populated
    net.node = torch.zeros(64, dtype=torch.float32, device="cuda")
    net.cdf = torch.zeros(65, dtype=torch.float64, device="cuda")
    node, cdf = (t.cpu().numpy().astype(np.float64) for t in net.build_grid())
    n = 2_000_000
    f, lq = net.sample(n, seed=9)
    f, lq = f.cpu().numpy(), lq.cpu().numpy()
    assert f.min() >= 0.0 and f.max() <= 1.0
    sub = np.random.default_rng(4).choice(n, 20000, replace=False)
    np.testing.assert_allclose(lq[sub], om.log_q(node, cdf, 4, f[sub]), atol=1e-9)
    # exact probability of each half-cell octant: P_c * sum_b d_b/S prod_a w_a,
    # w = 1/4 (lower half) or 3/4 (upper half) for the density 2t, mirrored for 2(1 - t)
    d = node.reshape(4, 4, 4)
    pc = np.diff(cdf) / cdf[-1]
    probs = np.zeros((64, 8))
    for c in range(64):
        i, j, k = c // 16, (c // 4) % 4, c % 4
        corners = [d[(i + (b >> 2 & 1)) % 4, (j + (b >> 1 & 1)) % 4, (k + (b & 1)) % 4] for b in range(8)]
        S = sum(corners)
        for o in range(8):
            half = [o >> 2 & 1, o >> 1 & 1, o & 1]
            tot = 0.0
            for b in range(8):
                bits = [b >> 2 & 1, b >> 1 & 1, b & 1]
                w = np.prod([(0.75 if h else 0.25) if bt else (0.25 if h else 0.75) for bt, h in zip(bits, half)])
                tot += corners[b] / S * w
            probs[c, o] = pc[c] * tot
    s = f * 4
    cell = np.clip(np.floor(s).astype(int), 0, 3)
    half = ((s - cell) >= 0.5).astype(int)
    idx = ((cell[:, 0] * 4 + cell[:, 1]) * 4 + cell[:, 2]) * 8 + half[:, 0] * 4 + half[:, 1] * 2 + half[:, 2]
    obs = np.bincount(idx, minlength=512)
    exp = probs.reshape(-1) * n
    chi2 = float(((obs - exp) ** 2 / exp).sum())
    assert abs(probs.sum() - 1) < 1e-12
    print("octant chi2 (511 dof):", chi2)
    assert chi2 < 511 + 6 * np.sqrt(2 * 511), chi2


def test_training_concentrates_the_density_on_the_data():
    net = _net(8)
    rng = np.random.default_rng(5)
    data = torch.as_tensor(_blob_data(200000, rng), device="cuda")
    losses = net.train(data, steps=300, batch=8192, lr=3e-3, log_every=50)
    assert losses[-1][1] < 0.6 * losses[0][1], losses
    net.build_grid()
    held = torch.as_tensor(_blob_data(20000, np.random.default_rng(6)), device="cuda")
    mean_lq = float(net.log_density(held).mean())
    # ln q of the two blobs (width 0.06 of the cell) averages ~ 3 nats for the true
    # density; a 16^3 grid and the 5 % floor keep part of it
    assert mean_lq > 1.5, mean_lq


@pytest.mark.parametrize("m,n,k", [(200, 100, 136), (384, 256, 512), (64, 64, 64), (1000, 256, 256)])
def test_gemm_bf16_row_major_operands(m, n, k):
    """bfloat16, K-contiguous operands (16-byte copies into shared memory): ragged M / N
    (zero-filled rows) and K not a multiple of the 64-wide K chunk."""
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(m * 7 + n + k)
    a = torch.randn(m, k, device="cuda", generator=g).bfloat16()
    b = torch.randn(n, k, device="cuda", generator=g).bfloat16()
    c = gemm(a, b)
    assert rel(c, a.float() @ b.float().T) < 1e-5


@pytest.mark.parametrize("m,n,k,split", [(256, 64, 3000, 2), (256, 64, 3000, 12), (300, 256, 1024, 1),
                                         (130, 128, 200, 1)])
def test_gemm_bf16_tma_ring_split_k_and_ragged(m, n, k, split):
    """bfloat16 operands with K contiguous take the TMA-fed kernel: K beyond the four-stage ring
    (stages refilled), split K (vector reductions into C), ragged M, K not a multiple of 64
    (zero-filled boxes), 64-, 128- and 256-wide tiles."""
    from kups_gb300.mlp import gemm

    g = torch.Generator(device="cuda").manual_seed(m + n + k + split)
    a = torch.randn(m, k, device="cuda", generator=g).bfloat16()
    b = torch.randn(n, k, device="cuda", generator=g).bfloat16()
    c = torch.zeros(m, n, device="cuda")
    gemm(a, b, c, beta=1.0 if split > 1 else 0.0, split_k=split)
    assert rel(c, a.float() @ b.float().T) < 1e-5
