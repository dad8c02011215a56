"""float64 numpy restatement of the tuner's cost model (csrc/kernels/mlp.cu):
3-layer MLP D -> 128 -> 128 -> 1 with ReLU, packed parameters W1, b1, W2, b2,
W3, b3, loss = mean squared error.  Test infrastructure: the checker of the
GPU forward pass and gradients."""
import numpy as np

D, H = 24, 128


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + H * D].reshape(H, D); o += H * D
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H].reshape(1, H); o += H
    b3 = p[o:o + 1]; o += 1
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0)
    H2 = np.maximum(H1 @ W2.T + b2, 0)
    return (H2 @ W3.T + b3)[:, 0], (X, H1, H2)


def loss_grad(p, X, y):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    pred, (X, H1, H2) = forward(p, X)
    n = len(y)
    e = pred - np.asarray(y, dtype=np.float64)
    loss = float(np.mean(e * e))
    dP = (2.0 * e / n)[:, None]
    gW3 = dP.T @ H2
    gb3 = dP.sum(0)
    dZ2 = (dP @ W3) * (H2 > 0)
    gW2 = dZ2.T @ H1
    gb2 = dZ2.sum(0)
    dZ1 = (dZ2 @ W2) * (H1 > 0)
    gW1 = dZ1.T @ X
    gb1 = dZ1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
