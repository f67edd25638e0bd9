"""FP64 restatement of the learned-guess MLP (12 -> 64 -> 64 -> 3, tanh). TEST INFRASTRUCTURE ONLY.

Forward pass, mean-squared loss over all outputs and its gradient, in the parameter
layout of the GPU kernels: W1[64][12], b1[64], W2[64][64], b2[64], W3[3][64], b3[3].
"""
import numpy as np

NF, NH, NO = 12, 64, 3


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    o = 0
    out = []
    for shape in ((NH, NF), (NH,), (NH, NH), (NH,), (NO, NH), (NO,)):
        n = int(np.prod(shape))
        out.append(w[o:o + n].reshape(shape))
        o += n
    return out


def loss_and_grad(w, X, Y):
    """Mean over samples and outputs of (f(x) - y)^2 and its gradient w.r.t. the parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    out = h2 @ W3.T + b3
    d = out - Y
    n = d.size
    loss = float(np.sum(d * d) / n)
    d3 = 2.0 * d / n
    gW3, gb3 = d3.T @ h2, d3.sum(0)
    d2 = (d3 @ W3) * (1 - h2 * h2)
    gW2, gb2 = d2.T @ h1, d2.sum(0)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    gW1, gb1 = d1.T @ X, d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
