"""IVFFlatIndex and TopKRouting, mirroring src/indices/ivf_flat.jl and
src/indices/multilevel/routing.jl (TopKRouting / select_indices).

Build and search run on the GPU through ``libmanngpu.so``: KMeans
(k-means++, Lloyd on a subsample, one full assignment) gives the centroids,
a stable grouping gives the inverted lists (ascending point ids per list, the
order of the reference's counting pass), and a query routes to its nprobe
nearest centroids and scans those lists in the FP32 form.

Layouts as in the rest of the package: ``data`` d x n (columns are points),
``Neighbor`` ids 1-based.  ``lists`` holds 1-based ids like the reference's
``Vector{Vector{Int}}``; the CSR arrays handed to the C ABI are 0-based.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .distances import Euclidean, Metric, SqEuclidean, default_distance, metric_code
from .indices import AbstractANNIndex, Neighbor, points_view


@dataclass
class IVFFlatIndex(AbstractANNIndex):
    """``IVFFlatIndex{T,Dm,Dc}`` (src/indices/ivf_flat.jl:12-20).  Centroids are
    d x nlist (columns), ``list_offsets``/``list_ids`` the 0-based CSR form of
    ``lists``; the data matrix is passed on every query."""
    centroids: np.ndarray
    centroid_norms: np.ndarray
    list_offsets: np.ndarray
    list_ids: np.ndarray
    dimension: int
    default_nprobe: int
    distance: Metric
    centroid_metric: Metric
    kmeans_iters: int = 0
    _device: dict = field(default_factory=dict, repr=False, compare=False)

    @property
    def nlist(self) -> int:
        return int(self.centroids.shape[1])

    @property
    def lists(self):
        """Per-list 1-based point ids (the reference's ``lists`` field)."""
        o = self.list_offsets
        return [(self.list_ids[o[c]:o[c + 1]].astype(np.int64) + 1).tolist() for c in range(self.nlist)]

    @classmethod
    def build(cls, data, *, nlist: int, nprobe: int = 10, distance: Metric = default_distance,
              centroid_metric: Metric = Euclidean(), kmeans_max_iters: int = 25,
              kmeans_tol: float = 1e-4, kmeans_subsample_size: int | None = -1, seed: int = 0):
        """``build_index(IVFFlatIndex, data; nlist, nprobe=10, distance, centroid_metric,
        kmeans_max_iters=25, kmeans_tol=1e-4, kmeans_subsample_size=max(256 nlist, 32768))``
        (src/indices/ivf_flat.jl:30-93).  ``kmeans_subsample_size=None`` fits on all points."""
        a = np.asarray(data)
        if a.ndim != 2 or a.shape[0] <= 0:
            raise ArgumentError("Dataset must have at least one dimension")
        d, n = int(a.shape[0]), int(a.shape[1])
        if n <= 0:
            raise ArgumentError("Dataset must contain at least one point")
        if nlist <= 0:
            raise ArgumentError("nlist must be positive")
        if not isinstance(centroid_metric, (Euclidean, SqEuclidean)):
            raise ArgumentError("centroid_metric must be Euclidean or SqEuclidean")
        metric_code(distance)
        if kmeans_subsample_size == -1:
            kmeans_subsample_size = max(256 * nlist, 32_768)
        X = points_view(a)
        C = np.empty((nlist, d), np.float32)
        offs = np.empty(nlist + 1, np.int64)
        ids = np.empty(n, np.int32)
        it = np.zeros(1, np.int32)
        p = _lib.IvfBuildParams(nlist, metric_code(centroid_metric), kmeans_max_iters, 0, kmeans_tol,
                                int(kmeans_subsample_size or 0), int(seed) & (2**64 - 1))
        _lib.check(_lib.load().mann_ivf_build(p, X.ctypes.data, n, d, C.ctypes.data, offs.ctypes.data,
                                              ids.ctypes.data, it.ctypes.data))
        Ct = np.asfortranarray(C.T)
        norms = (C.astype(np.float64) ** 2).sum(axis=1).astype(np.float32)
        return cls(Ct, norms, offs, ids, d, max(1, min(nprobe, nlist)), distance, centroid_metric,
                   int(it[0]))

    def save(self, path) -> None:
        """Write the index (centroids, norms, CSR lists, settings) to an .npz file."""
        from .distances import metric_code

        np.savez(path, format=np.array("manifoldann-gb300/ivf-flat/1"), centroids=self.centroids,
                 centroid_norms=self.centroid_norms, list_offsets=self.list_offsets, list_ids=self.list_ids,
                 dimension=np.int64(self.dimension), default_nprobe=np.int64(self.default_nprobe),
                 distance=np.int64(metric_code(self.distance)),
                 centroid_metric=np.int64(metric_code(self.centroid_metric)),
                 kmeans_iters=np.int64(self.kmeans_iters))

    @classmethod
    def load(cls, path):
        """Read an index written by ``save``."""
        from .distances import CosineDist

        metrics = {0: Euclidean, 1: SqEuclidean, 2: CosineDist}
        with np.load(path) as z:
            if str(z["format"]) != "manifoldann-gb300/ivf-flat/1":
                raise ArgumentError(f"not an IVF-Flat index file: {path}")
            return cls(np.asfortranarray(z["centroids"]), z["centroid_norms"].copy(), z["list_offsets"].copy(),
                       z["list_ids"].copy(), int(z["dimension"]), int(z["default_nprobe"]),
                       metrics[int(z["distance"])](), metrics[int(z["centroid_metric"])](), int(z["kmeans_iters"]))

    def _check(self, a: np.ndarray, qlen: int) -> None:
        """``_validate_dimensions`` (src/indices/ivf_flat.jl:95-101)."""
        if a.shape[0] != self.dimension:
            raise DimensionMismatch(f"Expected data with {self.dimension} rows")
        if qlen != self.dimension:
            raise DimensionMismatch(f"Expected query of length {self.dimension}")

    def search_arrays(self, data, queries, k: int, *, nprobe: int | None = None):
        """Batch search: (ids [q, k] 0-based int32 with -1 padding, dists [q, k])."""
        a = np.asarray(data)
        Q = np.asarray(queries)
        if Q.ndim == 1:
            Q = Q.reshape(-1, 1)
        self._check(a, Q.shape[0])
        nq = Q.shape[1]
        k = int(k)
        if k <= 0 or nq == 0:
            return np.empty((nq, 0), np.int32), np.empty((nq, 0), np.float32)
        nprobe = self.default_nprobe if nprobe is None else int(nprobe)
        nprobe = min(max(nprobe, 1), self.nlist)
        X = points_view(a)
        qs = points_view(Q)
        C = np.ascontiguousarray(self.centroids.T, dtype=np.float32)
        ids = np.empty((nq, k), np.int32)
        dists = np.empty((nq, k), np.float32)
        p = _lib.params(metric_code(self.distance), k, _lib.PREC_FP32, 0, 0)
        _lib.check(_lib.load().mann_ivf_search(
            p, nprobe, metric_code(self.centroid_metric), X.ctypes.data, X.shape[0], self.dimension,
            C.ctypes.data, self.nlist, self.list_offsets.ctypes.data, self.list_ids.ctypes.data,
            qs.ctypes.data, nq, ids.ctypes.data, dists.ctypes.data))
        return ids, dists

    def query(self, data, q, k: int, *, nprobe: int | None = None):
        """``query(index::IVFFlatIndex, data, q, k; nprobe=index.default_nprobe)``
        (src/indices/ivf_flat.jl:135-168): list of Neighbor (shorter than k when
        the probed lists hold fewer points); a d x m matrix gives a list of lists."""
        Q = np.asarray(q)
        if isinstance(q, (list, tuple)):
            if len(q) == 0:
                return []
            Q = np.stack([np.asarray(v) for v in q], axis=1)
        single = Q.ndim == 1
        ids, dists = self.search_arrays(data, Q, k, nprobe=nprobe)
        out = [[Neighbor(int(i) + 1, float(d)) for i, d in zip(ids[r], dists[r]) if i >= 0]
               for r in range(ids.shape[0])]
        return out[0] if single else out


def ivf_search_device(index: IVFFlatIndex, data_dev, queries_dev, k: int, nprobe: int, out_ids,
                      out_dists, stream: int = 0, centroids_dev=None, offsets_dev=None, ids_dev=None):
    """Search with device buffers (torch CUDA tensors or raw pointers): data
    [n][d] and queries [q][d] float32 row-major, outputs [q][k]."""
    def ptr(t):
        return t if isinstance(t, int) else t.data_ptr()

    n = data_dev.shape[0]
    nq = queries_dev.shape[0]
    p = _lib.params(metric_code(index.distance), int(k), _lib.PREC_FP32, 0, 0)
    _lib.check(_lib.load().mann_ivf_search_device(
        p, int(nprobe), metric_code(index.centroid_metric), ptr(data_dev), n, index.dimension,
        ptr(centroids_dev), index.nlist, ptr(offsets_dev), ptr(ids_dev), ptr(queries_dev), nq,
        ptr(out_ids), ptr(out_dists), stream))


@dataclass(frozen=True)
class TopKRouting:
    """``TopKRouting(k)`` (src/indices/multilevel/routing.jl:36-44): follow the k
    children with the smallest routing distances."""
    k: int

    def __post_init__(self):
        if self.k <= 0:
            raise ArgumentError("k must be positive")


def _order_keys(d: np.ndarray) -> np.ndarray:
    """Float32 -> uint32 keys whose unsigned order is the float order, NaN last
    and -0 before +0 (the order the GPU's top-k keys use)."""
    b = np.ascontiguousarray(d, np.float32).view(np.uint32)
    k = np.where(b >> 31 == 1, ~b, b | np.uint32(0x80000000)).astype(np.uint32)
    return np.where(np.isnan(d), np.uint32(0xFFFFFFFF), k)


def select_indices(policy, distances, indices):
    """``select_indices(::TopKRouting, assignment, indices)`` (routing.jl:94-118):
    1-based indices of the min(k, available) smallest of the first
    ``available = min(len(indices), len(distances))`` distances, ascending by
    (distance, index).  ``indices`` is the list of child indices or its length.
    For a LearnedProbeRouting the second argument is the query vector."""
    if not isinstance(policy, TopKRouting):
        from .probe import LearnedProbeRouting, select_indices_learned

        if isinstance(policy, LearnedProbeRouting):
            return select_indices_learned(policy, distances, indices)
        raise ArgumentError(f"no select_indices method for {type(policy).__name__}")
    n_children = indices if isinstance(indices, int) else len(indices)
    if n_children <= 0:
        return []
    d = np.asarray(getattr(distances, "distances", distances), np.float32).ravel()
    available = min(n_children, d.size)
    if available <= 0:
        raise ArgumentError("Transform produced no routing distances for TopKRouting")
    m = min(policy.k, available)
    order = np.lexsort((np.arange(available), _order_keys(d[:available])))
    return (order[:m] + 1).tolist()
