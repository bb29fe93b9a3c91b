"""The learned-proposal oracle checked against mathematics (it has no reference counterpart).

- the hand-derived backward pass against central finite differences of the
  float64 loss (relative 1e-6);
- the grid density integrates to one (two-point Gauss-Legendre per axis is
  exact for a trilinear function; 1e-12);
- the density is continuous across cell faces and across the periodic
  boundary (1e-9).
"""

import numpy as np

from oracle import mlp as om


def small_params(rng, scale=0.3):
    p = {k: rng.normal(0, scale / np.sqrt(s[-1]), s) for k, (o, s) in om.OFFSETS.items()}
    for k in ("b1", "b2", "b3", "b4"):
        p[k] = rng.normal(0, 0.1, p[k].shape)
    return p


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = small_params(rng)
    freq = rng.integers(-3, 4, (32, 3))
    x = rng.uniform(0, 1, (24, 3))
    y = (np.arange(24) < 12).astype(float)
    _, grads = om.loss_and_grad(p, x, y, freq, emulate=False)
    h = 1e-6
    for name in ("W1", "b1", "W2", "b2", "W3", "b3", "w4", "b4"):
        flat = p[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp, _ = om.loss_and_grad(p, x, y, freq, emulate=False)
            flat[idx] = old - h
            lm, _ = om.loss_and_grad(p, x, y, freq, emulate=False)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            an = grads[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 * max(1e-4, abs(fd)) + 1e-10, (name, idx, fd, an)


def test_grid_density_is_normalised():
    rng = np.random.default_rng(1)
    G = 5
    node = rng.uniform(0.05, 3.0, G**3)
    cdf = om.cdf_from_node(node, G)
    gl = np.array([0.5 - 0.5 / np.sqrt(3), 0.5 + 0.5 / np.sqrt(3)])
    pts = np.stack(np.meshgrid(gl, gl, gl, indexing="ij"), -1).reshape(-1, 3)
    cells = np.stack(np.meshgrid(*[np.arange(G)] * 3, indexing="ij"), -1).reshape(-1, 3)
    f = (cells[:, None, :] + pts[None]) / G
    q = np.exp(om.log_q(node, cdf, G, f.reshape(-1, 3)))
    integral = q.reshape(len(cells), 8).mean(1).sum() / G**3
    assert abs(integral - 1.0) < 1e-12


def test_grid_density_is_continuous_and_periodic():
    rng = np.random.default_rng(2)
    G = 6
    node = rng.uniform(0.05, 3.0, G**3)
    cdf = om.cdf_from_node(node, G)
    base = rng.uniform(0, 1, (50, 3))
    for a in range(3):
        for face in (2, G):  # an inner face and the periodic boundary
            lo, hi = base.copy(), base.copy()
            lo[:, a] = face / G - 1e-12
            hi[:, a] = face / G + 1e-12
            np.testing.assert_allclose(om.log_q(node, cdf, G, lo), om.log_q(node, cdf, G, hi), atol=1e-9)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-8, 1.0 + 2**-9, -2.5, 3.0e38])
    r = om.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2**-6 and r[3] == 1.0 and r[4] == -2.5
    assert np.isfinite(r[5])
