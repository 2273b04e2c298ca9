"""FP64 restatement of the learned coarse probe's forward and backward pass.

TEST INFRASTRUCTURE: imported only by tests/ (the checker of the GPU probe
kernels), never by the ``manifoldann_gb300`` package.

The probe has no counterpart in the reference (it is a routing strategy
beside TopKRouting, src/indices/multilevel/routing.jl:91-118), so nothing of
the reference pins it: this module is the mathematical definition, and its
own gradient is pinned by central finite differences (tests/test_probe_oracle.py).

Network: s = W3 g(W2 g(W1 x + b1) + b2) + b3 [- beta ||x - c||^2], g = GELU
(erf form), loss = mean over rows of softmax cross-entropy against the
distribution of the row's label lists.  ``bf16=True`` rounds to BF16 exactly
where the GPU kernels store BF16 (inputs, weights, hidden activations and the
back-propagated signals), with everything else in FP64.
"""
from __future__ import annotations

import math

import numpy as np

_SQRT1_2 = 1.0 / math.sqrt(2.0)
_INV_SQRT_2PI = 1.0 / math.sqrt(2.0 * math.pi)


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    x = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (x >> np.uint64(16)) & np.uint64(1)
    r = ((x + np.uint64(0x7FFF) + lsb) >> np.uint64(16)) << np.uint64(16)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _erf(z):
    from scipy.special import erf

    return erf(z)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z * _SQRT1_2))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z * _SQRT1_2)) + z * _INV_SQRT_2PI * np.exp(-0.5 * z * z)


def layout(din, h1, h2, nout):
    """Offsets of the flat parameter vector: W1 b1 W2 b2 W3 b3 theta."""
    o = {}
    p = 0
    for name, size in (("w1", h1 * din), ("b1", h1), ("w2", h2 * h1), ("b2", h2), ("w3", nout * h2),
                       ("b3", nout), ("theta", 1)):
        o[name] = (p, p + size)
        p += size
    o["total"] = p
    return o


def unpack(params, din, h1, h2, nout):
    L = layout(din, h1, h2, nout)
    P = np.asarray(params, np.float64)

    def g(n, shape=None):
        a, b = L[n]
        v = P[a:b]
        return v.reshape(shape) if shape else v

    return (g("w1", (h1, din)), g("b1"), g("w2", (h2, h1)), g("b2"), g("w3", (nout, h2)), g("b3"),
            float(g("theta")[0]))


def sqdist(X, C):
    X = np.asarray(X, np.float64)
    C = np.asarray(C, np.float64)
    return ((X[:, None, :] - C[None, :, :]) ** 2).sum(-1)


def label_dist(labels, nout):
    lab = np.asarray(labels)
    Y = np.zeros((lab.shape[0], nout))
    for r in range(lab.shape[0]):
        v = lab[r][(lab[r] >= 0) & (lab[r] < nout)]
        for c in v:
            Y[r, c] += 1.0 / len(v)
    return Y


def forward_backward(params, dims, X, labels, centroids=None, bf16_round=True):
    """Loss and flat gradient (FP64) of one batch; dims = (din, h1, h2, nout)."""
    din, h1, h2, nout = dims
    W1, b1, W2, b2, W3, b3, theta = unpack(params, *dims)
    r = bf16 if bf16_round else (lambda a: np.asarray(a, np.float64))
    Xb = r(X)
    W1b, W2b, W3b = r(W1), r(W2), r(W3)
    Z1 = Xb @ W1b.T + b1
    H1 = r(gelu(Z1))
    Z2 = H1 @ W2b.T + b2
    H2 = r(gelu(Z2))
    S = H2 @ W3b.T + b3
    beta = math.exp(theta)
    D = None
    if centroids is not None:
        D = sqdist(X, centroids)
        S = S - beta * D
    nb = S.shape[0]
    Y = label_dist(labels, nout)
    has = Y.sum(1) > 0
    m = S.max(1, keepdims=True)
    lse = (m + np.log(np.exp(S - m).sum(1, keepdims=True)))[:, 0]
    loss = float(np.where(has, lse - (Y * S).sum(1), 0.0).sum() / nb)
    P = np.exp(S - lse[:, None])
    G = np.where(has[:, None], (P - Y) / nb, 0.0)
    Gb = r(G)
    grads = {}
    grads["w3"] = Gb.T @ H2
    grads["b3"] = Gb.sum(0)
    dZ2 = r((Gb @ W3b) * gelu_grad(Z2))
    grads["w2"] = dZ2.T @ H1
    grads["b2"] = dZ2.sum(0)
    dZ1 = r((dZ2 @ W2b) * gelu_grad(Z1))
    grads["w1"] = dZ1.T @ Xb
    grads["b1"] = dZ1.sum(0)
    grads["theta"] = np.array([(G * (-beta * D)).sum() if D is not None else 0.0])
    L = layout(*dims)
    flat = np.zeros(L["total"])
    for k, v in grads.items():
        a, b = L[k]
        flat[a:b] = np.asarray(v).ravel()
    return loss, flat


def scores(params, dims, X, centroids=None, bf16_round=True):
    """Scores [n][nout] of the network (FP64, BF16 rounding as on the GPU)."""
    W1, b1, W2, b2, W3, b3, theta = unpack(params, *dims)
    r = bf16 if bf16_round else (lambda a: np.asarray(a, np.float64))
    H1 = r(gelu(r(X) @ r(W1).T + b1))
    H2 = r(gelu(H1 @ r(W2).T + b2))
    S = H2 @ r(W3).T + b3
    if centroids is not None:
        S = S - math.exp(theta) * sqdist(X, centroids)
    return S
