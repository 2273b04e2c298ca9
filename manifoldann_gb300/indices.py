"""BruteForceIndex and the generic query interface, mirroring the reference's
ANN-index API (src/ann_index.jl, src/indices/bruteforce.jl).

Data layout follows the reference: ``data`` is a d x n matrix whose columns
are the points (Julia ``Matrix{Float32}``); a query batch is d x q.  Ids in
``Neighbor`` are 1-based, as in Julia.  All arithmetic runs on the GPU in
Float32 (other element types are converted).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, NamedTuple

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .distances import Metric, default_distance, metric_code

PRECISIONS = {"fp32": _lib.PREC_FP32, "bf16": _lib.PREC_BF16, "fp8": _lib.PREC_FP8, "auto": _lib.PREC_AUTO,
              "fp16": _lib.PREC_FP16}


class Neighbor(NamedTuple):
    """``Neighbor{T}(id, dist)`` (src/utils/neighbor_heaps.jl:11-14); id is 1-based."""
    id: int
    dist: float


def neighbor_ids(neighbors):
    """``neighbor_ids`` (src/utils/neighbor_heaps.jl:22-44): ids of one list, or of each list."""
    if len(neighbors) and not isinstance(neighbors[0], Neighbor):
        return [neighbor_ids(n) for n in neighbors]
    return [n.id for n in neighbors]


class AbstractANNIndex:
    pass


@dataclass
class BruteForceIndex(AbstractANNIndex):
    """``BruteForceIndex{T,D}`` (src/indices/bruteforce.jl:16-20): metadata only --
    the caller passes the data matrix on every query."""
    dimension: int
    n_points: int
    distance: Metric


def points_view(data) -> np.ndarray:
    """d x n matrix (columns = points) -> row-major [n][d] float32 without a copy
    when ``data`` is already Fortran-ordered float32."""
    a = np.asarray(data)
    if a.ndim != 2:
        raise ArgumentError("data must be a d x n matrix")
    return np.ascontiguousarray(a.T, dtype=np.float32)


def index_distance(index) -> Metric:
    return index.distance


def supports_mutation(index) -> bool:
    return isinstance(index, BruteForceIndex)


def configured_k(index):
    """``configured_k`` (src/ann_index.jl:153): BruteForce exposes no default k."""
    return None


def build_index(cls, data, *, distance: Metric = default_distance, **kwargs):
    """``build_index(BruteForceIndex, data; distance)`` (src/indices/bruteforce.jl:31-35)."""
    if cls is BruteForceIndex:
        a = np.asarray(data)
        if a.ndim != 2 or a.shape[0] <= 0:
            raise ArgumentError("Dataset must have at least one dimension")
        if a.shape[1] <= 0:
            raise ArgumentError("Dataset must contain at least one point")
        metric_code(distance)
        return BruteForceIndex(int(a.shape[0]), int(a.shape[1]), distance)
    builder = getattr(cls, "build", None)
    if builder is None:
        raise ArgumentError(f"no build_index method for {cls}")
    return builder(data, distance=distance, **kwargs)


def insert(index: BruteForceIndex, points) -> BruteForceIndex:
    """``insert!`` (src/indices/bruteforce.jl:82-95): bookkeeping only."""
    a = np.asarray(points)
    if a.ndim == 1:
        if a.shape[0] != index.dimension:
            raise DimensionMismatch(f"Expected point dimension {index.dimension}")
        index.n_points += 1
        return index
    if a.shape[0] != index.dimension:
        raise DimensionMismatch(f"Expected point dimension {index.dimension}")
    index.n_points += int(a.shape[1])
    return index


class _ShapeOnly:
    """Stands in for a matrix of the given shape in the argument checks."""

    def __init__(self, shape):
        self.shape = tuple(shape)
        self.ndim = len(self.shape)


def _validate(index: BruteForceIndex, data: np.ndarray, qlen: int) -> None:
    """``validate_index_dimensions`` (src/utils/validation.jl:8-18)."""
    if data.shape[0] != index.dimension:
        raise DimensionMismatch(f"Expected data with {index.dimension} rows")
    if qlen != index.dimension:
        raise DimensionMismatch(f"Expected query length {index.dimension}")
    if data.shape[1] < index.n_points:
        raise ArgumentError(f"Data contains {data.shape[1]} points but index tracks {index.n_points}")


class DeviceDataset:
    """Device copy of a d x N point matrix (an owned ``mann_dataset*``).

    Searches given a DeviceDataset in place of the data matrix copy only
    their queries.  The copy does not follow later changes of the host
    matrix: call ``upload`` after ``insert`` (src/indices/bruteforce.jl:82-95)
    or any other change of the points."""

    def __init__(self, data):
        pts = points_view(np.asarray(data))
        self.n, self.d = int(pts.shape[0]), int(pts.shape[1])
        h = C.c_void_p()
        _lib.check(_lib.load().mann_dataset_create(pts.ctypes.data, self.n, self.d, C.byref(h)))
        self.handle = h

    @property
    def shape(self):
        """(d, N), the shape of the matrix it copies."""
        return (self.d, self.n)

    def upload(self, data) -> None:
        pts = points_view(np.asarray(data))
        if pts.shape[1] != self.d:
            raise DimensionMismatch(f"Expected points of dimension {self.d}, got {pts.shape[1]}")
        _lib.check(_lib.load().mann_dataset_upload(self.handle, pts.ctypes.data, int(pts.shape[0])))
        self.n = int(pts.shape[0])

    def close(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            _lib.load().mann_dataset_destroy(h)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def knn_arrays(index: BruteForceIndex, data, queries, k: int, *, precision: str = "fp32",
               fp64_ties: bool = False, margin: int = 0, report: bool = False, fp64_error: bool = False):
    """Batch exact kNN on the GPU; returns (ids [q, min(k,n)] 0-based int32,
    dists [q, min(k,n)] float32[, report dict]).  ``queries`` is d x q;
    ``data`` the d x N matrix or a DeviceDataset of it.
    With ``fp64_error`` the report's ``max_abs_err_fp64`` holds the largest
    |returned distance - FP64 distance| over all returned neighbours."""
    ds = data if isinstance(data, DeviceDataset) else None
    a = _ShapeOnly(ds.shape) if ds is not None else np.asarray(data)
    Q = np.asarray(queries)
    if Q.ndim == 1:
        Q = Q.reshape(-1, 1)
    if Q.shape[0] != a.shape[0]:
        raise DimensionMismatch(f"Expected queries with {a.shape[0]} rows, got {Q.shape[0]}")
    _validate(index, a, Q.shape[0])
    n = a.shape[1]
    nq = Q.shape[1]
    keff = min(int(k), n)
    if keff <= 0 or nq == 0:
        e = (np.empty((nq, 0), np.int32), np.empty((nq, 0), np.float32))
        return e + ({},) if report else e
    qs = points_view(Q)
    ids = np.empty((nq, keff), np.int32)
    dists = np.empty((nq, keff), np.float32)
    flags = (_lib.FLAG_FP64_TIES if fp64_ties else 0) | (_lib.FLAG_FP64_ERR if fp64_error else 0)
    p = _lib.params(metric_code(index.distance), keff, PRECISIONS[precision], margin, flags)
    rep = _lib.KnnReport()
    lib = _lib.load()
    if ds is not None:
        _lib.check(lib.mann_knn_dataset(p, ds.handle, qs.ctypes.data, nq, ids.ctypes.data, dists.ctypes.data,
                                        rep))
    else:
        base = points_view(a)
        _lib.check(lib.mann_knn(p, base.ctypes.data, n, qs.ctypes.data, nq, a.shape[0], ids.ctypes.data,
                                dists.ctypes.data, rep))
    if report:
        return ids, dists, rep.as_dict()
    return ids, dists


def _to_neighbors(ids_row, dists_row):
    return [Neighbor(int(i) + 1, float(d)) for i, d in zip(ids_row, dists_row) if i >= 0]


def query(index, data, q, k: int, **kwargs):
    """``query(index, data, q, k)``.

    * q a vector: one query (src/indices/bruteforce.jl:46-71) -> list of Neighbor;
    * q a d x m matrix: batch (src/ann_index.jl:71-101) -> list of lists;
    * q a list of vectors: stacked, then as a matrix (src/ann_index.jl:110-120).
    """
    if not isinstance(index, BruteForceIndex):
        return index.query(data, q, k, **kwargs)
    if isinstance(q, (list, tuple)):
        if len(q) == 0:
            return []
        q = np.stack([np.asarray(v) for v in q], axis=1)
    Q = np.asarray(q)
    a = np.asarray(data)
    if Q.ndim == 1:
        _validate(index, a, Q.shape[0])
        if min(int(k), a.shape[1]) <= 0:
            return []
        ids, dists = knn_arrays(index, a, Q.reshape(-1, 1), k, **kwargs)
        return _to_neighbors(ids[0], dists[0])
    if Q.shape[0] != a.shape[0]:
        raise DimensionMismatch(f"Expected queries with {a.shape[0]} rows, got {Q.shape[0]}")
    if Q.shape[1] == 0:
        return []
    ids, dists = knn_arrays(index, a, Q, k, **kwargs)
    return [_to_neighbors(ids[i], dists[i]) for i in range(ids.shape[0])]
