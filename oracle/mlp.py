"""Float64 restatement of the learned cost model's network, for checking the
GPU kernels (test infrastructure: only tests import it).

The network is the one stile_gb300/csrc/mlp.cu implements: F -> 64 -> 32 -> 1
with ReLU after the two hidden layers, parameters in one flat vector laid
out W1[F][64], b1[64], W2[64][32], b2[32], W3[32], b3.  The reference's
network (PyTorchMLP, my_cost_model.py:1010-1029) has the same hidden widths;
its loss for training is the mean squared error (MLP_train_cost_model.py:
81-204), as here.
"""
import numpy as np

F, H1, H2 = 12, 64, 32
N_PARAMS = F * H1 + H1 + H1 * H2 + H2 + H2 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    assert p.size == N_PARAMS
    o = 0
    W1 = p[o:o + F * H1].reshape(F, H1); o += F * H1
    b1 = p[o:o + H1]; o += H1
    W2 = p[o:o + H1 * H2].reshape(H1, H2); o += H1 * H2
    b2 = p[o:o + H2]; o += H2
    W3 = p[o:o + H2]; o += H2
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    return h2 @ W3 + b3


def loss_and_grad(p, x, t):
    """Mean squared error and its gradient with respect to the flat
    parameter vector."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    a1 = x @ W1 + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ W3 + b3
    d = y - t
    loss = float(np.sum(d * d) / n)
    dy = 2.0 * d / n
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    dh2 = np.outer(dy, W3) * (a2 > 0)
    gW2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (a1 > 0)
    gW1 = x.T @ dh1
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, g
