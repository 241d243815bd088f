"""CPU oracle of the learned tracklet scorer (TEST INFRASTRUCTURE ONLY).

Forward and backward of the 16-64-64-1 MLP in float64 with the rounding
points of the GPU kernels: the normalised input, the weights W1 and W2 and
the first hidden layer are rounded to BF16 (nearest even); everything else
is exact here (the kernels sum in FP32, so results agree to FP32 rounding of
the sums).  Loss: mean over the batch of
    pos_weight*y*softplus(-z) + (1-y)*softplus(z),  p = sigmoid(z).
Used by tests/ to check the GPU gradients and the tensor-core scores.
"""
import numpy as np


def bf16_round(x):
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.astype(np.uint32).view(np.float32)


def _split(params, nf=16, h=64):
    p = np.asarray(params, np.float64)
    o = 0
    w1 = p[o:o + h * nf].reshape(h, nf); o += h * nf
    b1 = p[o:o + h]; o += h
    w2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    w3 = p[o:o + h]; o += h
    return w1, b1, w2, b2, w3, p[o]


def forward(params, mean, inv_std, X, exact=False):
    """p (float64) and the intermediates of every row of X [n, 16].
    exact=True drops the BF16 roundings (to check the gradient formulas by
    finite differences)."""
    rnd = (lambda a: np.asarray(a, np.float64)) if exact else (
        lambda a: bf16_round(np.asarray(a, np.float32)).astype(np.float64))
    w1, b1, w2, b2, w3, b3 = _split(params)
    w1b = rnd(w1)
    w2b = rnd(w2)
    xn = (np.asarray(X, np.float32) - np.asarray(mean, np.float32)) * np.asarray(inv_std, np.float32)
    x = rnd(xn)
    a1 = x @ w1b.T + b1
    h1 = rnd(np.maximum(a1, 0))
    a2 = h1 @ w2b.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ w3 + b3
    p = 1.0 / (1.0 + np.exp(-z))
    return p, dict(x=x, a1=a1, h1=h1, a2=a2, h2=h2, z=z, w2b=w2b)


def softplus(a):
    return np.maximum(a, 0) + np.log1p(np.exp(-np.abs(a)))


def gradient(params, mean, inv_std, X, y, pos_weight, exact=False):
    """(gradient vector in the kernels' parameter order, loss).  The BF16
    roundings are passed straight through, as in the GPU kernel."""
    p, c = forward(params, mean, inv_std, X, exact)
    y = np.asarray(y, np.float64)
    n = len(y)
    z = c["z"]
    loss = np.sum(pos_weight * y * softplus(-z) + (1 - y) * softplus(z)) / n
    dz = (p * (pos_weight * y + 1 - y) - pos_weight * y) / n
    w1, b1, w2, b2, w3, b3 = _split(params)
    dh2 = (c["a2"] > 0) * dz[:, None] * w3[None, :]
    g_w3 = (dz[:, None] * c["h2"]).sum(0)
    g_b3 = dz.sum()
    g_w2 = dh2.T @ c["h1"]
    g_b2 = dh2.sum(0)
    dh1 = (c["a1"] > 0) * (dh2 @ c["w2b"])
    g_w1 = dh1.T @ c["x"]
    g_b1 = dh1.sum(0)
    g = np.concatenate([g_w1.reshape(-1), g_b1, g_w2.reshape(-1), g_b2, g_w3, [g_b3]])
    return g, loss
