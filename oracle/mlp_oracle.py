"""CPU restatement (numpy, FP64) of the warm-start MLP of
pdal_gb300/csrc/mlp.cu: the same parameter layout (W1 in x hidden row-major,
b1, W2, b2, W3, b3), ReLU hidden layers, linear output, mean squared error over
all outputs.  Test infrastructure only: the checker of the CUDA kernels'
forward pass and gradients."""
from __future__ import annotations

import numpy as np


def unpack(p: np.ndarray, inp: int, h: int, out: int):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + inp * h].reshape(inp, h); o += inp * h
    b1 = p[o:o + h]; o += h
    W2 = p[o:o + h * h].reshape(h, h); o += h * h
    b2 = p[o:o + h]; o += h
    W3 = p[o:o + h * out].reshape(h, out); o += h * out
    b3 = p[o:o + out]; o += out
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(p, X, inp, h, out):
    W1, b1, W2, b2, W3, b3 = unpack(p, inp, h, out)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(X @ W1 + b1, 0.0)
    H2 = np.maximum(H1 @ W2 + b2, 0.0)
    return H2 @ W3 + b3, (X, H1, H2)


def loss_grad(p, X, Y, inp, h, out):
    """(mean squared error, gradient in the parameter layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, inp, h, out)
    P, (X, H1, H2) = forward(p, X, inp, h, out)
    D = P - np.asarray(Y, dtype=np.float64)
    cnt = D.size
    loss = float((D * D).sum() / cnt)
    dP = 2.0 * D / cnt
    gW3 = H2.T @ dP
    gb3 = dP.sum(0)
    dH2 = (dP @ W3.T) * (H2 > 0)
    gW2 = H1.T @ dH2
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (H1 > 0)
    gW1 = X.T @ dH1
    gb1 = dH1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
