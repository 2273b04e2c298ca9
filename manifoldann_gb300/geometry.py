"""Local geometry over kNN neighbourhoods, mirroring src/geometry/pca.jl
(PCAMethod, PCAGeometry, fit_geometry, project, reconstruct, local_distance).

The fits run on the GPU (``mann_local_pca``): one call fits every centre of a
batch -- the per-node loop of build_weighted_graph
(src/graphs/weighted_knn_graph.jl:247-264) becomes one launch.  Ids are
1-based as in Julia; ``data`` is d x n.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .indices import points_view


@dataclass(frozen=True)
class PCAMethod:
    """``PCAMethod(; intrinsic_dim=nothing, min_variance_ratio=0.95)`` (pca.jl:44-57)."""
    intrinsic_dim: Optional[int] = None
    min_variance_ratio: float = 0.95

    def __post_init__(self):
        if self.intrinsic_dim is not None and self.intrinsic_dim < 1:
            raise ArgumentError(f"intrinsic_dim must be >= 1, got {self.intrinsic_dim}")
        if not (0.0 < self.min_variance_ratio <= 1.0):
            raise ArgumentError(f"min_variance_ratio must be in (0, 1], got {self.min_variance_ratio}")


@dataclass
class PCAGeometry:
    """``PCAGeometry{T}`` (pca.jl:79-83): centre [d], basis d x dim (orthonormal
    columns), eigenvalues [dim] (squared singular values, descending)."""
    center: np.ndarray
    basis: np.ndarray
    eigenvalues: np.ndarray


def intrinsic_dimension(geom: PCAGeometry) -> int:
    return int(geom.basis.shape[1])


def project(geom: PCAGeometry, x) -> np.ndarray:
    """Coordinates of x in the tangent space: basis^T (x - center)."""
    return geom.basis.T @ (np.asarray(x, np.float32) - geom.center)


def reconstruct(geom: PCAGeometry, y) -> np.ndarray:
    return geom.center + geom.basis @ np.asarray(y, np.float32)


def local_distance(geom: PCAGeometry, a, b) -> float:
    """``local_distance(::PCAGeometry, from, to)`` (pca.jl:255-259)."""
    return float(np.linalg.norm(project(geom, b) - project(geom, a)))


def fit_geometries(method: PCAMethod, data, neighbors, centers=None, query_points=None):
    """Batched fit: neighbors [m][k] 1-based ids (0 / negative = none, k <= 32),
    centres 1-based data ids [m] or query_points d x m.  Returns
    (dims [m], eigenvalues [m][maxd], bases [m][maxd][d]) with maxd = min(d, k)."""
    a = np.asarray(data)
    X = points_view(a)
    n, d = X.shape
    nb = np.asarray(neighbors)
    if nb.ndim != 2:
        raise ArgumentError("neighbors must be an m x k array")
    m, k = nb.shape
    if k > 32:
        raise ArgumentError("local PCA takes at most 32 neighbours per centre")
    nb0 = np.ascontiguousarray(np.where(nb > 0, nb - 1, -1), dtype=np.int32)
    cen = None
    qp = None
    if centers is not None:
        cen = np.ascontiguousarray(np.asarray(centers, np.int64) - 1, dtype=np.int32)
        if cen.shape != (m,):
            raise DimensionMismatch("centers must hold one id per row of neighbors")
    elif query_points is not None:
        qp = points_view(np.asarray(query_points).reshape(d, -1))
        if qp.shape[0] != m:
            raise DimensionMismatch("query_points must hold one point per row of neighbors")
    else:
        raise ArgumentError("give centers or query_points")
    maxd = max(1, min(d, k))
    dims = np.empty(m, np.int32)
    eig = np.empty((m, maxd), np.float32)
    basis = np.empty((m, maxd, d), np.float32)
    p = _lib.PcaParams(int(method.intrinsic_dim or 0), 0, float(method.min_variance_ratio))
    _lib.check(_lib.load().mann_local_pca(
        p, X.ctypes.data, n, d, cen.ctypes.data if cen is not None else None,
        qp.ctypes.data if qp is not None else None, m, nb0.ctypes.data, k, maxd, dims.ctypes.data,
        eig.ctypes.data, basis.ctypes.data))
    return dims, eig, basis


def fit_geometry(method: PCAMethod, data, center, neighbor_indices) -> PCAGeometry:
    """``fit_geometry(method::PCAMethod, data, center_idx | query_point,
    neighbor_indices)`` (pca.jl:101-126) for one centre."""
    a = np.asarray(data)
    nb = np.asarray(list(neighbor_indices), np.int64).reshape(1, -1)
    if np.isscalar(center) or np.asarray(center).ndim == 0:
        dims, eig, basis = fit_geometries(method, a, nb, centers=[int(center)])
        c = np.asarray(a[:, int(center) - 1], np.float32)
    else:
        c = np.asarray(center, np.float32)
        dims, eig, basis = fit_geometries(method, a, nb, query_points=c.reshape(-1, 1))
    dd = int(dims[0])
    return PCAGeometry(c, basis[0, :dd].T.copy(), eig[0, :dd].copy())


# ---------------------------------------------------------------- edge weights
class AbstractEdgeWeight:
    code = -1


class EuclideanChord(AbstractEdgeWeight):
    """``EuclideanChord()`` (src/graphs/edge_weight.jl:80): ||x_j - x_i||."""
    code = 0


class TangentProjectedSourceOnly(AbstractEdgeWeight):
    """``TangentProjectedSourceOnly()`` (edge_weight.jl:94)."""
    code = 1


class TangentProjectedSymmetricMean(AbstractEdgeWeight):
    """``TangentProjectedSymmetricMean()`` (edge_weight.jl:106)."""
    code = 2


class TangentProjectedSymmetricMax(AbstractEdgeWeight):
    """``TangentProjectedSymmetricMax()`` (edge_weight.jl:119)."""
    code = 3


class CurvatureFreeSymmetric(AbstractEdgeWeight):
    """``CurvatureFreeSymmetric()`` (edge_weight.jl:147): (8 d_E - d_T^(x) - d_T^(y)) / 6,
    the chord where that is negative (counted)."""
    code = 4


def compute_edge_weights(rule: AbstractEdgeWeight, data, neighbors, dims=None, bases=None):
    """Weights of every edge of a graph: neighbors [n][k] 1-based (0 = none ->
    NaN), tangent estimates (dims [n], bases [n][maxd][d] from fit_geometries)
    for the tangent rules.  Returns (weights [n][k] float32, negative fallbacks)."""
    import ctypes as C

    X = points_view(np.asarray(data))
    n, d = X.shape
    nb = np.asarray(neighbors)
    if nb.shape[0] != n:
        raise DimensionMismatch("one neighbour row per point")
    k = nb.shape[1]
    nb0 = np.ascontiguousarray(np.where(nb > 0, nb - 1, -1), dtype=np.int32)
    out = np.empty((n, k), np.float32)
    neg = C.c_int64(0)
    if rule.code != 0 and (dims is None or bases is None):
        raise ArgumentError(f"{type(rule).__name__} requires per-vertex tangent estimates; got `geometries=nothing`")
    dd = np.ascontiguousarray(dims, np.int32) if dims is not None else None
    bb = np.ascontiguousarray(bases, np.float32) if bases is not None else None
    maxd = int(bb.shape[1]) if bb is not None else 0
    _lib.check(_lib.load().mann_edge_weights(
        rule.code, X.ctypes.data, n, d, nb0.ctypes.data, k, dd.ctypes.data if dd is not None else None,
        bb.ctypes.data if bb is not None else None, maxd, out.ctypes.data, C.byref(neg)))
    return out, int(neg.value)


# ---------------------------------------------------------------- weighted graphs
def candidate_neighbors(index, data, candidate_k: int) -> np.ndarray:
    """The candidate lists of ``build_weighted_graph_with_candidates``
    (src/graphs/weighted_knn_graph.jl:497-524): for every node i the 1-based ids
    of ``query(index, data, x_i, candidate_k + 1)`` without i, the first
    ``candidate_k`` of them (``_candidates(i)``, :502-509).  That is the kNN
    graph's own rule (_prepare_neighbors), so all nodes come from one batched
    self-graph search instead of one query per node.  Returns [n][candidate_k]."""
    from .graphs import knn_graph_arrays

    ids, _ = knn_graph_arrays(index, data, int(candidate_k))
    return ids.astype(np.int64) + 1


@dataclass
class WeightedKNNGraph:
    """``WeightedKNNGraph`` (src/graphs/weighted_knn_graph.jl): the kNN graph
    (0-based ids [n][k] and distances), every node's fitted geometry in the
    batched form of ``fit_geometries`` (dims [n], eigenvalues [n][maxd], bases
    [n][maxd][d]) and the edge weights [n][k]."""
    graph_ids: np.ndarray
    graph_dists: np.ndarray
    dims: np.ndarray
    eigenvalues: np.ndarray
    bases: np.ndarray
    edge_weights: np.ndarray
    negative_fallbacks: int


def build_weighted_graph(method: PCAMethod, index, data, *, k: int, candidate_k: Optional[int] = None,
                         edge_weight: AbstractEdgeWeight = TangentProjectedSourceOnly()) -> WeightedKNNGraph:
    """``build_weighted_graph(method, index, data; k, candidate_k, edge_weight)``
    (weighted_knn_graph.jl:432-463) with ``NoSharing``: the kNN graph with k
    neighbours; every node's geometry fitted on its graph neighbours, or on its
    candidate_k candidates when candidate_k > k (:455-461, :482-524); then the
    edge weights of the graph's edges (:194-236).  Each step is one batched
    GPU call over all nodes."""
    from .graphs import knn_graph_arrays

    gi, gd = knn_graph_arrays(index, data, int(k))
    n = gi.shape[0]
    if candidate_k is None or candidate_k <= k:
        nbrs = gi.astype(np.int64) + 1
    else:
        nbrs = candidate_neighbors(index, data, candidate_k)
    dims, eig, bases = fit_geometries(method, data, nbrs, centers=np.arange(n) + 1)
    w, neg = compute_edge_weights(edge_weight, data, gi.astype(np.int64) + 1, dims, bases)
    return WeightedKNNGraph(gi, gd, dims, eig, bases, w, neg)
