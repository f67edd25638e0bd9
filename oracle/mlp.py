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


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(w, X, bf16_operands=False):
    """Network outputs for feature rows X; with bf16_operands the GEMM operands (features and
    hidden activations) are rounded to BF16 first, as the tensor-core kernels store them."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    r = bf16 if bf16_operands else (lambda a: np.asarray(a, np.float64))
    h1 = r(np.tanh(r(X) @ W1.T + b1))
    h2 = r(np.tanh(h1 @ W2.T + b2))
    return h2 @ W3.T + b3


def loss_and_grad(w, X, Y, bf16_operands=False):
    """Mean over samples and outputs of (f(x) - y)^2 and its gradient w.r.t. the parameters.
    With bf16_operands, every GEMM operand the tensor-core training kernel stores as BF16 is
    rounded first: the features, the hidden activations (also in the tanh derivatives), the
    output error in the layer-3 weight gradient and both back-propagated deltas."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    r = bf16 if bf16_operands else (lambda a: np.asarray(a, np.float64))
    X = r(X)
    h1 = r(np.tanh(X @ W1.T + b1))
    h2 = r(np.tanh(h1 @ W2.T + b2))
    out = h2 @ W3.T + b3
    d = out - Y
    n = d.size
    loss = float(np.sum(d * d) / n)
    d3 = 2.0 * d / n
    gW3, gb3 = r(d3).T @ h2, r(d3).sum(0)
    d2 = r((d3 @ W3) * (1 - h2 * h2))
    gW2, gb2 = d2.T @ h1, d2.sum(0)
    d1 = r((d2 @ W2) * (1 - h1 * h1))
    gW1, gb1 = d1.T @ X, d1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
