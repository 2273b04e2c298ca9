"""kNN-graph materialisation, mirroring src/graphs/knn_graph.jl.

``build_knn_graph`` issues ONE library call for the whole graph instead of
the reference's serial column loop (knn_graph.jl:63-67); the self-drop rule of
``_prepare_neighbors`` (:105-130) runs inside the library.  Symmetrisation
and metadata follow the reference (:76-80, :171-210).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError
from .distances import metric_code
from .indices import PRECISIONS, BruteForceIndex, DeviceDataset, _validate, configured_k, points_view


@dataclass
class KNNGraph:
    """``KNNGraph{I,M}`` (src/graphs/knn_graph.jl:9-14); neighbour ids are 1-based."""
    neighbors: list
    k: int
    include_self: bool
    metadata: Any = None

    def __len__(self):
        return len(self.neighbors)

    def __getitem__(self, i):
        return self.neighbors[i]

    def __iter__(self):
        return iter(self.neighbors)


def _resolve_graph_k(index, k):
    """``_resolve_graph_k`` (src/graphs/knn_graph.jl:83-103)."""
    configured = configured_k(index)
    if k is None:
        if configured is None:
            raise ArgumentError(f"Index {type(index).__name__} does not expose a default k; pass `k=` explicitly")
        return configured
    if k <= 0:
        raise ArgumentError("k must be positive")
    if configured is not None and k > configured:
        raise ArgumentError(f"Requested k={k} exceeds index configuration k={configured}")
    return int(k)


def _symmetrize_adjacency(adjacency, n_points):
    """``_symmetrize_adjacency`` (src/graphs/knn_graph.jl:196-210): union of i->j and j->i, sorted."""
    sym = [set() for _ in range(n_points)]
    for i, nbrs in enumerate(adjacency):
        for j in nbrs:
            sym[i].add(j)
            sym[j - 1].add(i + 1)
    return [sorted(s) for s in sym]


def _create_graph_metadata(original_k, directed, node_metadata, n_points):
    """``_create_graph_metadata`` (src/graphs/knn_graph.jl:171-184)."""
    stored = None
    if node_metadata is not None:
        if len(node_metadata) != n_points:
            raise ArgumentError(
                f"Metadata length {len(node_metadata)} must equal number of points {n_points}")
        stored = list(node_metadata)
    return {"original_k": original_k, "directed": directed, "node_metadata": stored}


def knn_graph_arrays(index: BruteForceIndex, data, k: int, *, include_self: bool = False,
                     precision: str = "fp32", fp64_ties: bool = False, margin: int = 0,
                     report: bool = False, fp64_error: bool = False):
    """Self-kNN graph on the GPU: (ids [n, k] 0-based int32, dists [n, k]);
    ``data`` is the d x n matrix or a DeviceDataset of it.  With
    ``fp64_error`` the report's ``max_abs_err_fp64`` holds the largest
    |returned distance - FP64 distance| over all returned neighbours."""
    ds = data if isinstance(data, DeviceDataset) else None
    a = None if ds is not None else np.asarray(data)
    n = ds.n if ds is not None else a.shape[1]
    max_neighbors = n - (0 if include_self else 1)
    if not (0 < k <= max_neighbors):
        raise ArgumentError(f"k must satisfy 0 < k <= {max_neighbors} for dataset with {n} points")
    ids = np.empty((n, k), np.int32)
    dists = np.empty((n, k), np.float32)
    p = _lib.params(metric_code(index.distance), k, PRECISIONS[precision], margin,
                    (_lib.FLAG_FP64_TIES if fp64_ties else 0) | (_lib.FLAG_FP64_ERR if fp64_error else 0))
    rep = _lib.KnnReport()
    if ds is not None:
        _lib.check(_lib.load().mann_knn_graph_dataset(p, ds.handle, int(bool(include_self)), ids.ctypes.data,
                                                      dists.ctypes.data, rep))
    else:
        pts = points_view(a)
        _lib.check(_lib.load().mann_knn_graph(p, pts.ctypes.data, n, a.shape[0], int(bool(include_self)),
                                              ids.ctypes.data, dists.ctypes.data, rep))
    if report:
        return ids, dists, rep.as_dict()
    return ids, dists


def knn_graph_batched_arrays(clouds, k: int, *, distance=None, include_self: bool = False,
                             report: bool = False, precision: str = "fp32"):
    """Self-kNN graphs of many point sets (each d x n_i) in one library call:
    (ids [sum n_i, k] 0-based ids local to each set, dists, offsets [nsets+1]).
    ``precision="bf16"``: the tensor-core form (one segmented pass over every
    set, exact FP32 rerank; the same answer, k + 1 <= 24)."""
    from .distances import default_distance

    mats = [np.asarray(c) for c in clouds]
    if not mats:
        raise ArgumentError("at least one point set is needed")
    d = mats[0].shape[0]
    if any(m.ndim != 2 or m.shape[0] != d for m in mats):
        raise ArgumentError("all point sets must be d x n_i matrices of one d")
    offs = np.zeros(len(mats) + 1, np.int64)
    offs[1:] = np.cumsum([m.shape[1] for m in mats])
    pts = np.ascontiguousarray(np.concatenate([m.T for m in mats], axis=0), dtype=np.float32)
    N = int(offs[-1])
    ids = np.empty((N, k), np.int32)
    dists = np.empty((N, k), np.float32)
    p = _lib.params(metric_code(distance or default_distance), k, PRECISIONS[precision])
    rep = _lib.KnnReport()
    _lib.check(_lib.load().mann_knn_graph_batched(p, pts.ctypes.data, offs.ctypes.data, len(mats), d,
                                                  int(bool(include_self)), ids.ctypes.data, dists.ctypes.data,
                                                  rep))
    if report:
        return ids, dists, offs, rep.as_dict()
    return ids, dists, offs


def build_knn_graphs(clouds, *, k: int, distance=None, include_self: bool = False) -> list:
    """``build_knn_graph(build_index(BruteForceIndex, c; distance), c; k, include_self)``
    for every point set c, as one batched call; a list of KNNGraph."""
    ids, _, offs = knn_graph_batched_arrays(clouds, k, distance=distance, include_self=include_self)
    out = []
    for c in range(len(offs) - 1):
        block = ids[offs[c]:offs[c + 1]]
        adjacency = [[int(j) + 1 for j in row] for row in block]
        out.append(KNNGraph(adjacency, k, include_self,
                            _create_graph_metadata(k, True, None, int(offs[c + 1] - offs[c]))))
    return out


def knn_graph_symmetrize_csr(ids):
    """Union (undirected) graph of a kNN id table [n][k] (0-based, -1 = none) on
    the GPU as CSR: (row_offsets [n+1] int64, cols [nnz] int32 ascending per row)."""
    import ctypes as C

    a = np.ascontiguousarray(ids, dtype=np.int32)
    n, k = a.shape
    offs = np.empty(n + 1, np.int64)
    cols = np.empty(max(2 * n * k, 1), np.int32)
    nnz = C.c_int64(0)
    _lib.check(_lib.load().mann_knn_graph_symmetrize(a.ctypes.data, n, k, offs.ctypes.data, cols.ctypes.data,
                                                     C.byref(nnz)))
    return offs, cols[:nnz.value].copy()


def build_knn_graph(index, data, *, k: Optional[int] = None, include_self: bool = False,
                    directed: bool = True, metadata=None, **query_kwargs) -> KNNGraph:
    """``build_knn_graph(index, data; k, include_self, directed, metadata)``
    (src/graphs/knn_graph.jl:42-81)."""
    a = np.asarray(data)
    n_points = a.shape[1]
    if n_points <= 0:
        raise ArgumentError("Dataset must contain at least one point")
    resolved_k = _resolve_graph_k(index, k)
    max_neighbors = n_points - (0 if include_self else 1)
    if not (0 < resolved_k <= max_neighbors):
        raise ArgumentError(
            f"k must satisfy 0 < k <= {max_neighbors} for dataset with {n_points} points")
    if isinstance(index, BruteForceIndex):
        _validate(index, a, a.shape[0])
        ids, _ = knn_graph_arrays(index, a, resolved_k, include_self=include_self, **query_kwargs)
        adjacency = [[int(j) + 1 for j in row] for row in ids]
    else:
        adjacency = index.build_adjacency(a, resolved_k, include_self, **query_kwargs)
    original_k = resolved_k
    if not directed:
        if isinstance(index, BruteForceIndex):
            offs, cols = knn_graph_symmetrize_csr(ids)
            adjacency = [(cols[offs[i]:offs[i + 1]].astype(np.int64) + 1).tolist() for i in range(n_points)]
        else:
            adjacency = _symmetrize_adjacency(adjacency, n_points)
        resolved_k = max(len(nb) for nb in adjacency)
    meta = _create_graph_metadata(original_k, directed, metadata, n_points)
    return KNNGraph(adjacency, resolved_k, include_self, meta)


def has_metadata(graph: KNNGraph) -> bool:
    return graph.metadata is not None and graph.metadata["node_metadata"] is not None


def graph_metadata(graph: KNNGraph):
    return graph.metadata


def node_metadata(graph: KNNGraph, i: int):
    """1-based, as the reference (src/graphs/knn_graph.jl:214-220)."""
    if graph.metadata is None:
        raise ArgumentError("Graph does not store metadata")
    if graph.metadata["node_metadata"] is None:
        raise ArgumentError("Graph does not store node-level metadata")
    return graph.metadata["node_metadata"][i - 1]
