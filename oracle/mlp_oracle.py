"""TEST INFRASTRUCTURE ONLY: float64 reference of the surrogate MLP's loss gradients.

Same network as ci_mlp (cppimpact_gb300/csrc/ci_mlp.cu): Z1 = X W1 + b1, H1 = tanh(Z1),
Z2 = H1 W2 + b2, H2 = tanh(Z2), Y = H2 W3 + b3, loss = mean((Y - T)^2); the flat
parameter vector is W1, b1, W2, b2, W3, b3 (row-major).  Reverse-mode derivatives
written out by hand.
"""
import numpy as np


def unpack(p, n_in, H, n_out):
    p = np.asarray(p, dtype=np.float64)
    sizes = [n_in * H, H, H * H, H, H * n_out, n_out]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(n_in, H), b1, W2.reshape(H, H), b2, W3.reshape(H, n_out), b3


def loss_and_grad(p, X, T, n_in, H, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, H, n_out)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    H1 = np.tanh(X @ W1 + b1)
    H2 = np.tanh(H1 @ W2 + b2)
    Y = H2 @ W3 + b3
    n = Y.size
    loss = np.sum((Y - T) ** 2) / n
    dY = 2.0 * (Y - T) / n
    gW3, gb3 = H2.T @ dY, dY.sum(0)
    dZ2 = (dY @ W3.T) * (1 - H2 ** 2)
    gW2, gb2 = H1.T @ dZ2, dZ2.sum(0)
    dZ1 = (dZ2 @ W2.T) * (1 - H1 ** 2)
    gW1, gb1 = X.T @ dZ1, dZ1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
