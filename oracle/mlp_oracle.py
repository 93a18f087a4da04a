"""Host restatement of the control-variate network (test infrastructure only:
imported by tests/, never by the package).

The network is the engine's exchange-energy model, csrc/k_mlp.cu:
  z1 = W1 x + b1, h1 = gelu(z1), z2 = W2 h1 + b2, h2 = gelu(z2), y = w3.h2 + b3,
gelu(z) = z Phi(z), loss = mean (y - t)^2 / 2, Adam with bias correction.
Parameters: W1 (H x F), b1 (H), W2 (H x H), b2 (H), w3 (H), b3 (1) flattened.
There is no reference counterpart (the reference has no learned part)."""
import numpy as np
from scipy.special import erf


def unpack(p, F, H):
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(p, x, H):
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, np.float64), x.shape[1], H)
    z1 = x @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    return h2 @ w3 + b3, (z1, h1, z2, h2)


def loss_and_grad(p, x, t, H):
    """(loss, flat gradient) of mean (y - t)^2 / 2."""
    F = x.shape[1]
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, np.float64), F, H)
    y, (z1, h1, z2, h2) = forward(p, x, H)
    B = x.shape[0]
    d = (y - t) / B
    gw3 = h2.T @ d
    gb3 = d.sum()
    dz2 = np.outer(d, w3) * gelu_d(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_d(z1)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    loss = 0.5 * np.mean((y - t) ** 2)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])


def adam(p, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
