"""FP64 CPU restatement of the warm-start MLP and its features (numpy).

TEST INFRASTRUCTURE ONLY.  Mirrors cumf_sgd_gb300/csrc/mlp.cu: parameters flattened as
W1[h][d_in], b1, W2[h][h], b2, W3[d_out][h], b3; GELU in the tanh form; loss = mean over rows
of the squared error summed over outputs."""
from __future__ import annotations

import numpy as np

C_GELU = 0.7978845608028654


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C_GELU * (1 + 3 * 0.044715 * x * x)


def unpack(params, d_in, h, d_out):
    p = np.asarray(params, dtype=np.float64)
    o = 0
    out = []
    for shape in ((h, d_in), (h,), (h, h), (h,), (d_out, h), (d_out,)):
        size = int(np.prod(shape))
        out.append(p[o:o + size].reshape(shape))
        o += size
    return out


def forward_backward(params, X, T, d_in, h, d_out):
    """Returns (loss, grads flattened) in float64."""
    W1, b1, W2, b2, W3, b3 = unpack(params, d_in, h, d_out)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    B = X.shape[0]
    z1 = X @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    a2 = gelu(z2)
    y = a2 @ W3.T + b3
    d = y - T
    loss = float((d * d).sum() / B)
    dy = 2 * d / B
    gW3 = dy.T @ a2
    gb3 = dy.sum(0)
    dz2 = (dy @ W3) * gelu_grad(z2)
    gW2 = dz2.T @ a1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


def bf16(x):
    """float64 -> float32 -> bfloat16 (round to nearest even), returned as float64: the
    rounding the GPU applies where it stores a bf16 operand (__float2bfloat16_rn)."""
    b = np.ascontiguousarray(np.asarray(x, np.float64).astype(np.float32)).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_backward_bf16(params, X, T, d_in, h, d_out, mistake=None):
    """forward_backward with the GPU's bf16 roundings applied where mlp.cu stores bf16
    operands (X, the weight copies, H1, H2, dY, dZ2, dZ1; pre-activations, Y and the products'
    accumulation stay wide), in float64 otherwise.  The GPU then differs from it only by fp32
    accumulation order and by the odd value that lands on the other side of a bf16 rounding
    boundary.  `mistake` plants a silent transposition (test use only): "gW2_transposed"
    returns dW2 transposed, "dH1_uses_W2T" back-propagates through W2 instead of W2^T."""
    W1, b1, W2, b2, W3, b3 = unpack(params, d_in, h, d_out)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    B = X.shape[0]
    xb, w1, w2, w3 = bf16(X), bf16(W1), bf16(W2), bf16(W3)
    z1 = xb @ w1.T + b1
    a1 = bf16(gelu(z1))
    z2 = a1 @ w2.T + b2
    a2 = bf16(gelu(z2))
    y = a2 @ w3.T + b3
    d = y - T
    loss = float((d * d).sum() / B)
    dy = bf16(2 * d / B)
    gW3 = dy.T @ a2
    gb3 = dy.sum(0)
    dz2 = bf16((dy @ w3) * gelu_grad(z2))
    gW2 = dz2.T @ a1
    if mistake == "gW2_transposed":
        gW2 = gW2.T
    gb2 = dz2.sum(0)
    dz1 = bf16((dz2 @ (w2.T if mistake == "dH1_uses_W2T" else w2)) * gelu_grad(z1))
    gW1 = dz1.T @ xb
    gb1 = dz1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])


GRAD_NAMES = ("W1", "b1", "W2", "b2", "W3", "b3")


def rel_err(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-30))


def gradient_bounds(params, X, T, d_in, h, d_out, slack=2e-3):
    """Per-tensor bounds for a GPU gradient against the FP64 restatement, derived from the bf16
    roundings: the distance between the bf16-rounded restatement and the exact one, times 2,
    plus `slack` for fp32 accumulation.  Returns (bf16 loss, bf16 grads, exact grads, bounds)."""
    l16, g16 = forward_backward_bf16(params, X, T, d_in, h, d_out)
    _, g64 = forward_backward(params, X, T, d_in, h, d_out)
    parts16, parts64 = unpack(g16, d_in, h, d_out), unpack(g64, d_in, h, d_out)
    bounds = {n: 2 * rel_err(a, b) + slack for n, a, b in zip(GRAD_NAMES, parts16, parts64)}
    return l16, g16, g64, bounds


def user_features(records, Q, m, k):
    """Features of users 0..m-1 (see cumf_user_features): rating-centred mean of the rated
    items' factors, log-degree, rating mean and variance; float64."""
    u = records["u"].astype(np.int64)
    v = records["v"].astype(np.int64)
    r = records["r"].astype(np.float64)
    deg = np.bincount(u, minlength=m).astype(np.float64)
    s1 = np.bincount(u, weights=r, minlength=m)
    s2 = np.bincount(u, weights=r * r, minlength=m)
    mean = np.divide(s1, deg, out=np.zeros(m), where=deg > 0)
    var = np.maximum(np.divide(s2, deg, out=np.zeros(m), where=deg > 0) - mean ** 2, 0)
    X = np.zeros((m, k + 3))
    c = (r - mean[u]) / deg[u]
    np.add.at(X[:, :k], u, c[:, None] * Q[v].astype(np.float64))
    X[:, k] = np.log1p(deg) / 4
    X[:, k + 1] = np.where(deg > 0, (mean - 3) / 2, 0)
    X[:, k + 2] = var / 2
    return X
