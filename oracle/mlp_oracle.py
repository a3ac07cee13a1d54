"""CPU ORACLE for the learned profile's network — test infrastructure only.

A numpy restatement, in float64, of the 16 -> 64 -> 64 (GELU) -> 2 network of
sampling-graph-mining_gb300/csrc/zg_mlp.cu: the same parameter layout, BF16 (round to nearest
even) working weights, exact-erf GELU, mean-squared-error loss and its analytic gradient, and
one Adam step.  Used to check the device forward, backward and optimiser kernels.
"""
import numpy as np
from scipy.special import erf

IN, H, OUT = 16, 64, 2
OW1 = 0
OB1 = OW1 + H * IN
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + OUT * H
NP = OB3 + OUT


def bf16(x):
    """float32 -> bfloat16 -> float32, round to nearest even."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params):
    w = bf16(params).astype(np.float64)
    return (w[OW1:OB1].reshape(H, IN), w[OB1:OW2], w[OW2:OB2].reshape(H, H), w[OB2:OW3],
            w[OW3:OB3].reshape(OUT, H), w[OB3:NP])


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = unpack(params)
    X = np.asarray(X, np.float64)
    z1 = X @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    return h2 @ W3.T + b3, (X, z1, h1, z2, h2)


def loss_and_grad(params, X, Y):
    W1, b1, W2, b2, W3, b3 = unpack(params)
    y, (X, z1, h1, z2, h2) = forward(params, X)
    Y = np.asarray(Y, np.float64)
    B = len(X)
    d = y - Y
    loss = float(np.mean(d * d))
    dy = 2.0 * d / (B * OUT)
    dz2 = (dy @ W3) * gelu_grad(z2)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    g = np.zeros(NP)
    g[OW1:OB1] = (dz1.T @ X).ravel()
    g[OB1:OW2] = dz1.sum(0)
    g[OW2:OB2] = (dz2.T @ h1).ravel()
    g[OB2:OW3] = dz2.sum(0)
    g[OW3:OB3] = (dy.T @ h2).ravel()
    g[OB3:NP] = dy.sum(0)
    return loss, g


def adam_step(params, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = params - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, m, v
