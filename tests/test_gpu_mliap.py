"""Local MLIAP on the GPU neighbour list against the float64 oracle: energies (rtol 1e-12),
dE/dx and dE/dtril against oracle central differences (1e-6 of the largest component),
and the incremental update against a full recomputation (rtol 1e-12), for the reference
test model and a nonlinear message network, on batched triclinic systems with images."""

import numpy as np
import pytest
import torch

from oracle import mliap as oml

pytestmark = pytest.mark.gpu


def torch_simple_model():
    emb = torch.full((3, 4), 0.1, dtype=torch.float64, device="cuda")
    w = torch.full((4, 1), 0.1, dtype=torch.float64, device="cuda")
    return (lambda z: emb[z], lambda h1, h2, d: h2 / (d.norm(dim=-1, keepdim=True) + 1.0),
            lambda h, m: ((h + m) @ w).squeeze(-1))


def mlp_models(seed=0, f=6):
    rng = np.random.default_rng(seed)
    emb = rng.normal(0, 0.5, (3, f))
    w1 = rng.normal(0, 0.4, (2 * f + 1, 8))
    w2 = rng.normal(0, 0.4, (8, f))
    wr = rng.normal(0, 0.3, (2 * f,))

    def make(xp, tanh, cat, as_arr):
        E, W1, W2, WR = (as_arr(a) for a in (emb, w1, w2, wr))

        def edge(h1, h2, d):
            r = (d * d).sum(-1, keepdims=True) ** 0.5 if xp is np else d.norm(dim=-1, keepdim=True)
            x = cat([h1 * h2, h2, r], -1)
            return tanh(x @ W1) @ W2 * (1.0 - r / 5.0) ** 2

        return (lambda z: E[z], edge, lambda h, m: tanh(cat([h, m], -1)) @ WR)

    npm = make(np, np.tanh, lambda xs, a: np.concatenate(xs, a), lambda a: a)
    tm = make(torch, torch.tanh, lambda xs, a: torch.cat(xs, a),
              lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda"))
    return npm, tm


def case(seed=1, S=2, N=50):
    rng = np.random.default_rng(seed)
    tril = np.array([[9.0, 0.8, 8.0, -0.7, 0.5, 8.5], [8.5, 0.0, 9.0, 0.6, -0.4, 9.5]])[:S]
    pos = rng.uniform(0, 8, (S * N, 3))
    z = rng.integers(0, 3, S * N)
    system = np.repeat(np.arange(S), N)
    return pos, z, system, tril, np.full(S, 5.0)


@pytest.mark.parametrize("which", ["reference_test_model", "mlp"])
def test_energy_and_gradients_match_oracle(which):
    from kups_gb300 import mliap

    pos, z, system, tril, cut = case()
    if which == "mlp":
        npm, tm = mlp_models()
    else:
        npm, tm = oml.simple_model(), torch_simple_model()
    pot = mliap.LocalMLIAP(*tm)
    res = pot.energy(pos, z, system, tril, cut)
    e_ref, h_ref, m_ref = oml.local_mliap_energy(npm, pos, z, system, tril, cut)
    np.testing.assert_allclose(res.energy.cpu().numpy(), e_ref, rtol=1e-12)
    np.testing.assert_allclose(res.cache.msg_sum.cpu().numpy(), m_ref, rtol=1e-11, atol=1e-14)
    g = res.grad.cpu().numpy()
    gt = res.grad_tril.cpu().numpy()
    h = 1e-6
    fd = np.zeros((8, 3))
    for k, i in enumerate(range(0, len(pos), len(pos) // 8)[:8]):
        for a in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[i, a] += h
            p2[i, a] -= h
            fd[k, a] = (oml.local_mliap_energy(npm, p1, z, system, tril, cut)[0].sum()
                        - oml.local_mliap_energy(npm, p2, z, system, tril, cut)[0].sum()) / (2 * h)
    rows = list(range(0, len(pos), len(pos) // 8))[:8]
    np.testing.assert_allclose(g[rows], fd, rtol=0, atol=1e-6 * max(np.abs(g).max(), 1e-3))
    fdt = np.zeros_like(gt)
    for s in range(len(tril)):
        for k in range(6):
            t1, t2 = tril.copy(), tril.copy()
            t1[s, k] += h
            t2[s, k] -= h
            fdt[s, k] = (oml.local_mliap_energy(npm, pos, z, system, t1, cut)[0][s]
                         - oml.local_mliap_energy(npm, pos, z, system, t2, cut)[0][s]) / (2 * h)
    np.testing.assert_allclose(gt, fdt, rtol=0, atol=1e-6 * max(np.abs(gt).max(), 1e-3))


def test_incremental_update_equals_full_recomputation():
    from kups_gb300 import mliap

    pos, z, system, tril, cut = case(seed=4)
    _, tm = mlp_models(seed=2)
    pot = mliap.LocalMLIAP(*tm)
    old = pot.energy(pos, z, system, tril, cut, gradients=False)
    rng = np.random.default_rng(7)
    changed = np.array([3, 17, 60])
    new_pos = pos.copy()
    new_pos[changed] += rng.normal(0, 1.5, (3, 3))  # large enough to change neighbour sets
    new_z = z.copy()
    new_z[17] = (z[17] + 1) % 3
    upd = pot.energy_update(old.cache, pos, new_pos, z, new_z, changed, system, tril, cut)
    full = pot.energy(new_pos, new_z, system, tril, cut, gradients=False)
    np.testing.assert_allclose(upd.energy.cpu().numpy(), full.energy.cpu().numpy(), rtol=1e-12)
    np.testing.assert_allclose(upd.cache.msg_sum.cpu().numpy(), full.cache.msg_sum.cpu().numpy(), rtol=1e-10,
                               atol=1e-13)
    assert not np.allclose(upd.energy.cpu().numpy(), old.energy.cpu().numpy())
