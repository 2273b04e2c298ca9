"""FP64 restatement of the reference's local PCA fit.

TEST INFRASTRUCTURE: imported only by tests/ (the checker of the GPU local
PCA), never by the ``manifoldann_gb300`` package.

Follows _fit_pca_geometry / _pca_eigen / _determine_dimension
(src/geometry/pca.jl:127-241): centre the neighbours on the centre point,
eigen-decompose the smaller of C^T C (d <= k) and C C^T (d > k, principal
directions back-projected as C w / sqrt(lambda)), eigenvalues descending and
clamped at zero, dimension fixed or the first cumulative share >= the ratio.
"""
from __future__ import annotations

import numpy as np


def fit_pca(center, neighbors, intrinsic_dim=None, min_variance_ratio=0.95):
    """center [d], neighbors [k][d] -> (dim, eigenvalues [dim], basis [d][dim])."""
    center = np.asarray(center, np.float64)
    nb = np.asarray(neighbors, np.float64)
    d = center.size
    k = nb.shape[0]
    if k < 2:
        dd = min(intrinsic_dim or 1, d)
        basis = np.zeros((d, dd))
        basis[np.arange(dd), np.arange(dd)] = 1.0
        return dd, np.ones(dd), basis
    C = (nb - center).T  # d x k, columns are centred neighbours
    if d <= k:
        vals, vecs = np.linalg.eigh(C @ C.T)
        vals = vals[::-1].clip(min=0.0)
        vecs = vecs[:, ::-1]
    else:
        vals, W = np.linalg.eigh(C.T @ C)
        vals = vals[::-1].clip(min=0.0)
        W = W[:, ::-1]
        tol = np.finfo(np.float32).eps * max(vals[0], 1.0) * max(d, k)
        vecs = np.zeros((d, k))
        for j in range(k):
            if vals[j] > tol:
                vecs[:, j] = C @ W[:, j] / np.sqrt(vals[j])
            elif j < d:
                vecs[j, j] = 1.0
    max_d = min(len(vals), d)
    if intrinsic_dim:
        dim = min(intrinsic_dim, max_d)
    elif vals.size == 0 or not np.any(vals):
        dim = 1
    else:
        total = vals.sum()
        cum = np.cumsum(vals) / total
        hit = np.nonzero(cum >= min_variance_ratio)[0]
        dim = int(hit[0]) + 1 if hit.size else max_d
    return dim, vals[:dim], vecs[:, :dim]


def edge_weights(rule, X, nbrs, bases, dims):
    """FP64 compute_edge_weight for every edge (src/graphs/edge_weight.jl:163-262):
    rule 0 chord, 1 source tangent, 2 mean, 3 max, 4 curvature-free (chord when
    negative).  bases[i] is d x dim_i.  Returns (weights [n][k], negatives)."""
    X = np.asarray(X, np.float64)
    n, k = nbrs.shape
    out = np.full((n, k), np.nan)
    neg = 0
    for i in range(n):
        for e in range(k):
            j = nbrs[i, e]
            if j < 0:
                continue
            diff = X[j] - X[i]
            dE = np.linalg.norm(diff)
            if rule == 0:
                out[i, e] = dE
                continue
            dx = np.linalg.norm(bases[i][:, :dims[i]].T @ diff)
            if rule == 1:
                out[i, e] = dx
                continue
            dy = np.linalg.norm(bases[j][:, :dims[j]].T @ diff)
            if rule == 2:
                out[i, e] = 0.5 * (dx + dy)
            elif rule == 3:
                out[i, e] = max(dx, dy)
            else:
                raw = (8 * dE - dx - dy) / 6
                if raw < 0:
                    out[i, e] = dE
                    neg += 1
                else:
                    out[i, e] = raw
    return out, neg
