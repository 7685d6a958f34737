"""ORACLE — test infrastructure, not the product.

NumPy restatement of the learned probe network's forward and backward passes
(puck_gb300/csrc/probe.cu), used to check the GPU gradients. The network has no
counterpart in the reference; this file is the definition it is checked against.

    Z1 = X W1^T + b1, H1 = GELU(Z1); Z2 = H1 W2^T + b2, H2 = GELU(Z2);
    Z = H2 W3^T + b3; loss = mean_i CE(softmax(Z_i), p_i),
    p_i = distribution of the query's label ids (0xFFFFFFFF = none).

With bf16=True every matrix product takes its two operands rounded to BF16
(round to nearest even), as the tensor-core contraction does, and accumulates
in float64; with bf16=False everything is float64.
"""
import math

import numpy as np

NO_LABEL = 0xFFFFFFFF


def to_bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _erf(x):
    return np.vectorize(math.erf, otypes=[np.float64])(x)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    cdf = 0.5 * (1.0 + _erf(x / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)
    return cdf + x * pdf


def split_params(flat, d, h, C):
    sizes = [(h, d), (h,), (h, h), (h,), (C, h), (C,)]
    out, o = [], 0
    for sh in sizes:
        m = int(np.prod(sh))
        out.append(np.asarray(flat[o:o + m], np.float64).reshape(sh))
        o += m
    return out


def targets(labels, C):
    n, L = labels.shape
    p = np.zeros((n, C))
    for i in range(n):
        ids = [int(c) for c in labels[i] if int(c) != NO_LABEL and int(c) < C]
        for c in ids:
            p[i, c] += 1.0 / len(ids)
    return p


def forward_backward(params, X, labels, d, h, C, bf16=True):
    """Returns (loss, flat gradient in the parameter layout)."""
    W1, b1, W2, b2, W3, b3 = split_params(params, d, h, C)
    r = (lambda a: to_bf16(a).astype(np.float64)) if bf16 else (lambda a: np.asarray(a, np.float64))
    X = np.asarray(X, np.float32)
    n = X.shape[0]
    Z1 = r(X) @ r(W1).T + b1
    H1 = gelu(Z1)
    Z2 = r(H1) @ r(W2).T + b2
    H2 = gelu(Z2)
    Z = r(H2) @ r(W3).T + b3
    m = Z.max(1, keepdims=True)
    lse = m + np.log(np.exp(Z - m).sum(1, keepdims=True))
    sm = np.exp(Z - lse)
    p = targets(labels, C)
    loss = float((p * (lse - Z)).sum() / n)
    dZ = (sm - p) / n
    gW3 = r(dZ).T @ r(H2)
    gb3 = dZ.sum(0)
    dZ2 = (r(dZ) @ r(W3)) * gelu_grad(Z2)
    gW2 = r(dZ2).T @ r(H1)
    gb2 = dZ2.sum(0)
    dZ1 = (r(dZ2) @ r(W2)) * gelu_grad(Z1)
    gW1 = r(dZ1).T @ r(X)
    gb1 = dZ1.sum(0)
    flat = np.concatenate([g.reshape(-1) for g in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, flat
