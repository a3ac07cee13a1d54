"""Pins the CPU oracle of the learned profile's network: its analytic gradient equals central
finite differences of its own loss (weights perturbed before BF16 rounding is bypassed by
perturbing in float64 on the unpacked network)."""
import numpy as np

import mlp_oracle as M


def _loss64(w64, X, Y):
    W1 = w64[M.OW1:M.OB1].reshape(M.H, M.IN)
    b1 = w64[M.OB1:M.OW2]
    W2 = w64[M.OW2:M.OB2].reshape(M.H, M.H)
    b2 = w64[M.OB2:M.OW3]
    W3 = w64[M.OW3:M.OB3].reshape(M.OUT, M.H)
    b3 = w64[M.OB3:M.NP]
    h1 = M.gelu(X @ W1.T + b1)
    h2 = M.gelu(h1 @ W2.T + b2)
    y = h2 @ W3.T + b3
    return np.mean((y - Y) ** 2)


def test_oracle_gradient_is_the_loss_derivative():
    rng = np.random.default_rng(0)
    params = (rng.normal(size=M.NP) * 0.2).astype(np.float32)
    params = M.bf16(params)  # exactly representable, so unpack() does not move them
    X = rng.normal(size=(9, 16))
    Y = rng.normal(size=(9, 2))
    loss, g = M.loss_and_grad(params, X, Y)
    w64 = params.astype(np.float64)
    assert abs(loss - _loss64(w64, X, Y)) < 1e-12
    idx = rng.choice(M.NP, size=60, replace=False)
    for i in idx:
        h = 1e-6
        wp, wm = w64.copy(), w64.copy()
        wp[i] += h
        wm[i] -= h
        fd = (_loss64(wp, X, Y) - _loss64(wm, X, Y)) / (2 * h)
        assert abs(fd - g[i]) < 1e-6 + 1e-5 * abs(g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.0078125, 1.01171875, -2.5e-3, 3.0e38], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == 1.015625
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)
