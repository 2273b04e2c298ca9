"""KMeansTransform and the KMeans helpers, mirroring
src/transforms/KMeansTransform.jl and src/transforms/kmeans/*.jl.

Matrices follow the reference: data d x n (columns are points), centroids
d x k.  Cluster ids returned by the Julia-named functions are 1-based, as in
Julia; the *_arrays helpers return 0-based ids.  All arithmetic runs on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError
from .distances import Euclidean, Metric, SqEuclidean, metric_code
from .indices import points_view

KMEANS_DEFAULT_MAX_ITERATIONS = 100  # src/utils/constants.jl:127
KMEANS_DEFAULT_TOLERANCE = 1e-6      # src/utils/constants.jl:135


@dataclass
class KMeansAssignment:
    """``KMeansAssignment`` (src/transforms/KMeansTransform.jl:85-87): distances to every centroid."""
    distances: np.ndarray


@dataclass
class TransformResult:
    data: np.ndarray
    assignment: KMeansAssignment


def _as_rows(a) -> np.ndarray:
    return points_view(a)


def pairwise_distances(X, centroids, distance: Metric) -> np.ndarray:
    """``pairwise_distances!`` (distance.jl:28-46): D k x n with D[i, j] = dist(centroid i, point j)."""
    Xr, Cr = _as_rows(X), _as_rows(centroids)
    if Xr.shape[1] != Cr.shape[1]:
        raise _lib.DimensionMismatch("Centroids must be d x k")
    n, k = Xr.shape[0], Cr.shape[0]
    D = np.empty((n, k), np.float32)
    _lib.check(_lib.load().mann_pairwise_distances(Xr.ctypes.data, n, Cr.ctypes.data, k, Xr.shape[1],
                                                   metric_code(distance), D.ctypes.data))
    return D.T  # k x n view with the reference's orientation


def assign_arrays(X, centroids, distance: Metric):
    """Exact nearest centroid of every point: (0-based ids int32 [n], distances [n])."""
    Xr, Cr = _as_rows(X), _as_rows(centroids)
    n, k = Xr.shape[0], Cr.shape[0]
    a = np.empty(n, np.int32)
    dist = np.empty(n, np.float32)
    _lib.check(_lib.load().mann_kmeans_assign(Xr.ctypes.data, n, Cr.ctypes.data, k, Xr.shape[1],
                                              metric_code(distance), a.ctypes.data, dist.ctypes.data))
    return a, dist


def assign_clusters(X, centroids, distance: Metric = Euclidean()):
    """``assign_clusters!`` (distance.jl:287-310) computed from the points: 1-based ids."""
    a, _ = assign_arrays(X, centroids, distance)
    return a.astype(np.int64) + 1


def init_kmeans_plus_plus(X, k: int, *, first: int, u) -> np.ndarray:
    """``init_kmeans_plus_plus`` (init.jl:56-102) with the caller's draws:
    `first` (1-based point index) and u[i] in [0,1) for i = 2..k (u[0] unused).
    Returns the d x k centroid matrix."""
    Xr = _as_rows(X)
    n, d = Xr.shape
    if not (0 < k <= n):
        raise ArgumentError(f"Cannot initialize {k} clusters with only {n} points")
    u = np.ascontiguousarray(u, dtype=np.float64)
    if u.size < k:
        raise ArgumentError("need k draws")
    idx = np.empty(k, np.int64)
    _lib.check(_lib.load().mann_kmeanspp(Xr.ctypes.data, n, d, k, int(first) - 1, u.ctypes.data,
                                         idx.ctypes.data))
    return np.ascontiguousarray(Xr[idx].T), idx + 1


def lloyd(centroids, X, distance: Metric, *, max_iters=KMEANS_DEFAULT_MAX_ITERATIONS,
          tol=KMEANS_DEFAULT_TOLERANCE):
    """``lloyd!`` (lloyd.jl:36-134): (centroids d x k, 1-based assignments, iterations)."""
    Xr, Cr = _as_rows(X), np.array(_as_rows(centroids), dtype=np.float32, copy=True)
    n, d = Xr.shape
    k = Cr.shape[0]
    a = np.empty(n, np.int32)
    it = np.zeros(1, np.int32)
    _lib.check(_lib.load().mann_kmeans_lloyd(Xr.ctypes.data, n, d, k, Cr.ctypes.data, max_iters, tol,
                                             metric_code(distance), a.ctypes.data, it.ctypes.data))
    return np.ascontiguousarray(Cr.T), a.astype(np.int64) + 1, int(it[0])


class KMeansTransform:
    """``KMeansTransform`` (src/transforms/KMeansTransform.jl:41-74)."""

    def __init__(self, *, k: int, distance: Metric, init: str = "kmeans_plus_plus",
                 max_iters: int = KMEANS_DEFAULT_MAX_ITERATIONS, tol: float = KMEANS_DEFAULT_TOLERANCE,
                 subsample_size: Optional[int] = None, centroid_type=np.float32):
        if k <= 0:
            raise ArgumentError("Number of clusters must be positive")
        if init not in ("random", "kmeans_plus_plus"):
            raise ArgumentError("init must be :random or :kmeans_plus_plus")
        if max_iters <= 0:
            raise ArgumentError("max_iters must be positive")
        if tol <= 0:
            raise ArgumentError("tol must be positive")
        if subsample_size is not None and subsample_size <= 0:
            raise ArgumentError("subsample_size must be positive or nothing")
        if not isinstance(distance, (Euclidean, SqEuclidean)):
            raise ArgumentError("KMeansTransform on the GPU supports Euclidean() and SqEuclidean()")
        self.k = k
        self.distance = distance
        self.init = init
        self.max_iters = max_iters
        self.tol = tol
        self.subsample_size = subsample_size
        self.centroid_type = centroid_type
        self.centroids = None       # d x k
        self.centroid_norms = None  # k
        self.pending_assignments = None  # 1-based
        self.iterations = 0


def fit(t: KMeansTransform, X, *, seed: int = 0) -> KMeansTransform:
    """``fit!(t, X; rng)`` (KMeansTransform.jl:106-161).  `seed` drives the
    library's own generator (Julia's RNG streams are not reproduced)."""
    Xr = _as_rows(X)
    n, d = Xr.shape
    if t.k > n:
        raise ArgumentError(f"Cannot fit {t.k} clusters with only {n} points")
    p = _lib.KmeansParams()
    p.k = t.k
    p.metric = metric_code(t.distance)
    p.init = 1 if t.init == "kmeans_plus_plus" else 0
    p.max_iters = t.max_iters
    p.tol = t.tol
    p.subsample = t.subsample_size or 0
    p.seed = seed
    C = np.empty((t.k, d), np.float32)
    a = np.empty(n, np.int32)
    it = np.zeros(1, np.int32)
    _lib.check(_lib.load().mann_kmeans_fit(p, Xr.ctypes.data, n, d, C.ctypes.data, a.ctypes.data,
                                           it.ctypes.data))
    t.centroids = np.ascontiguousarray(C.T.astype(t.centroid_type))
    t.centroid_norms = (C.astype(np.float64) ** 2).sum(1).astype(t.centroid_type)
    t.pending_assignments = a.astype(np.int64) + 1
    t.iterations = int(it[0])
    return t


def transform(t: KMeansTransform, x) -> TransformResult:
    """``transform(t, x)`` (KMeansTransform.jl:181-190): distances to all centroids."""
    if t.centroids is None:
        raise ArgumentError("KMeansTransform must be fitted before transforming")
    xv = np.asarray(x, dtype=np.float32).reshape(-1, 1)
    D = pairwise_distances(xv, t.centroids, t.distance)
    return TransformResult(np.asarray(x), KMeansAssignment(np.asarray(D[:, 0])))


def take_pending_assignments(t: KMeansTransform):
    """``take_pending_assignments!`` (KMeansTransform.jl:192-196)."""
    a = t.pending_assignments
    t.pending_assignments = None
    return a


def get_bucket_assignment(assignment: KMeansAssignment) -> int:
    """``get_bucket_assignment`` (src/transforms/utils.jl:41-43): 1-based arg-min (first minimum)."""
    return int(np.argmin(assignment.distances)) + 1
