"""TEST INFRASTRUCTURE ONLY: float64 numpy restatement of the cost-model MLP.

The schedule cost model (fftj.jl_gb300/csrc/mlp.cu) has no counterpart in
FFTJ.jl; this file restates its mathematics so that the GPU kernels'
forward pass and gradients can be checked on the CPU. Only tests/ import it.

Model: x (D) -> h1 = relu(W1 x + b1) (64) -> h2 = relu(W2 h1 + b2) (64)
-> f = w3 . h2 + b3. Loss: mean over rows of (f - y)^2. Parameters are
flattened as W1[64][D], b1[64], W2[64][64], b2[64], w3[64], b3.
"""
import numpy as np

H = 64


def layout(D):
    sizes = [("W1", H * D), ("b1", H), ("W2", H * H), ("b2", H), ("w3", H), ("b3", 1)]
    out, off = {}, 0
    for name, n in sizes:
        out[name] = (off, n)
        off += n
    return out, off


def unpack(params, D):
    lay, total = layout(D)
    p = np.asarray(params, dtype=np.float64)
    assert p.size == total
    g = {k: p[o:o + n] for k, (o, n) in lay.items()}
    return g["W1"].reshape(H, D), g["b1"], g["W2"].reshape(H, H), g["b2"], g["w3"], g["b3"][0]


def forward(params, X):
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(params, X.shape[1])
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    return h2 @ w3 + b3


def loss_and_grad(params, X, y):
    """Mean squared error and its gradient (flattened like params)."""
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n, D = X.shape
    W1, b1, W2, b2, w3, b3 = unpack(params, D)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    f = h2 @ w3 + b3
    e = f - y
    loss = float(np.mean(e * e))
    dout = 2 * e / n
    gw3 = h2.T @ dout
    gb3 = dout.sum()
    d2 = np.outer(dout, w3) * (a2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (a1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, grad
