"""CPU oracle of the learned opening criterion's network -- test infrastructure only.

The 5-64-64-1 ReLU network of include/tcgpu.h (parameters W1[64][5], b1[64], W2[64][64],
b2[64], w3[64], b3): forward pass, the mean-squared-error gradient in float64 (the check
for the GPU training kernel), and an emulation of the traversal's FP16 evaluation (weights
and hidden activations rounded to FP16, FP32 accumulation).
"""
import numpy as np

NIN, NH = 5, 64
NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1


def unpack(p):
    p = np.asarray(p)
    o = 0
    W1 = p[o:o + NH * NIN].reshape(NH, NIN); o += NH * NIN
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1.T + b1, 0.)
    h2 = np.maximum(h1 @ W2.T + b2, 0.)
    return h2 @ w3 + b3


def grad(p, x, t):
    """Gradient of mean((y - t)^2) with respect to the parameters, and the loss."""
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    a1 = x @ W1.T + b1
    h1 = np.maximum(a1, 0.)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0.)
    y = h2 @ w3 + b3
    e = y - t
    dy = 2. * e / n
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    d2 = np.outer(dy, w3) * (a2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ x
    gb1 = d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return g, float((e * e).mean())


def infer_fp16(p, x):
    """The traversal's evaluation: FP16 inputs, weights and hidden activations, FP32 sums."""
    W1, b1, W2, b2, w3, b3 = unpack(np.asarray(p, dtype=np.float32))
    h = lambda a: np.asarray(a, dtype=np.float16).astype(np.float32)
    x16 = h(x)
    a1 = x16 @ h(W1).T + b1.astype(np.float32)
    h1 = h(np.maximum(a1, 0.))
    a2 = h1 @ h(W2).T + b2.astype(np.float32)
    h2 = np.maximum(a2, 0.)
    return (h2 @ w3.astype(np.float32) + np.float32(b3)).astype(np.float32)
