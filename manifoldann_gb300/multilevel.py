"""MultiLevelIndex over a KMeans transform with BruteForce children, mirroring
the reference's multi-level API (src/indices/multilevel/): configs
(config.jl), TransformedIndex (transformed.jl:40-76), MultiLevelIndex
(multilevel.jl:44-56), the builder (builder.jl:61-218), single and batch
queries (query.jl:25-106, 279-474) and the merge strategies (merge.jl:79-169).

The batch query keeps the reference's inverted loop -- route every query,
group the queries by probed child, one batched search per child, map local
ids to global ids, merge per query -- with the searches on the GPU:

* ``engine="per_child"``: the points are copied to the device once per batch,
  grouped by child (each child's points contiguous), and every probed child
  gets one ``mann_knn_device`` call with its sub-batch of queries (the
  reference's one ``query(child, child_data, Q_sub, k)`` per child,
  query.jl:441-474);
* ``engine="scan"``: all probed children in one ``mann_ivf_scan_device``
  launch (the children are disjoint BruteForce partitions of the same data,
  so this is the per-child search followed by a (distance, id) merge).

Routing: the KMeans transform's distances to every centroid
(``mann_pairwise_distances``, FP32 difference form) and ``select_indices``
of the routing strategy (TopKRouting: the nprobe smallest, ties to the lower
child).  Ids are 1-based in ``Neighbor``; data is d x n.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .distances import Metric, default_distance, metric_code
from .indices import AbstractANNIndex, BruteForceIndex, Neighbor, build_index, points_view
from .ivf import TopKRouting, _order_keys, select_indices
from .transforms import KMeansTransform, fit, pairwise_distances


# ---------------------------------------------------------------- configs
@dataclass(frozen=True)
class TerminalConfig:
    """``TerminalConfig(index_type, params)`` (config.jl:37-45): a leaf index."""
    index_type: type = BruteForceIndex
    params: dict = field(default_factory=dict)


@dataclass(frozen=True)
class TransformedConfig:
    """``TransformedConfig(transform, routing, child_config)`` (config.jl:47-80).
    The transform is a prototype: the builder fits a fresh copy."""
    transform: KMeansTransform
    routing: Any
    child_config: TerminalConfig = field(default_factory=TerminalConfig)


# ---------------------------------------------------------------- merges
class SimpleMerge:
    """``SimpleMerge()`` (merge.jl:40): every child's neighbours, stable sort by
    distance, first occurrence of each id, the first k."""


class DisjointMerge:
    """``DisjointMerge()`` (merge.jl:150): children with disjoint points; a
    bounded max-heap of the k best, then sorted by (distance, id)."""


def _heap_push(heap, cap, nb):
    # BoundedMaxHeap push! (src/utils/neighbor_heaps.jl:84-104, sift :156-190):
    # max-heap on the distance alone, strict < admission when full
    if len(heap) < cap:
        heap.append(nb)
        i = len(heap) - 1
        while i > 0:
            p = (i - 1) >> 1
            if heap[i].dist > heap[p].dist:
                heap[i], heap[p] = heap[p], heap[i]
                i = p
            else:
                break
        return
    if nb.dist < heap[0].dist:
        heap[0] = nb
        i, n = 0, len(heap)
        while True:
            l, r, big = 2 * i + 1, 2 * i + 2, i
            if l < n and heap[l].dist > heap[big].dist:
                big = l
            if r < n and heap[r].dist > heap[big].dist:
                big = r
            if big == i:
                break
            heap[i], heap[big] = heap[big], heap[i]
            i = big


def merge_results(strategy, result_lists, k: int):
    """``merge_results(strategy, result_lists, k)`` (merge.jl:79-124, 150-169)."""
    total = sum(len(r) for r in result_lists)
    if total == 0:
        return []
    cap = min(int(k), total)
    if isinstance(strategy, DisjointMerge):
        heap: list = []
        for r in result_lists:
            for nb in r:
                _heap_push(heap, cap, nb)
        return sorted(heap, key=lambda nb: (nb.dist, nb.id))
    if not isinstance(strategy, SimpleMerge):
        raise ArgumentError(f"no merge_results method for {type(strategy).__name__}")
    allnb = sorted((nb for r in result_lists for nb in r), key=lambda nb: nb.dist)  # stable
    out, seen = [], set()
    for nb in allnb:
        if nb.id in seen:
            continue
        seen.add(nb.id)
        out.append(nb)
        if len(out) >= cap:
            break
    return out


# ---------------------------------------------------------------- index types
@dataclass
class TransformedIndex(AbstractANNIndex):
    """``TransformedIndex(transform, routing_strategy, indices, id_mappings,
    child_data, bucket_lookup)`` (transformed.jl:40-76).  ``id_mappings[c]`` are
    the 1-based parent ids of child c's points (bucketed transforms);
    ``bucket_lookup[b]`` is the 1-based child position of bucket b (0 = empty)."""
    transform: Any
    routing_strategy: Any
    indices: list
    id_mappings: Optional[list] = None
    child_data: Optional[list] = None
    bucket_lookup: Optional[np.ndarray] = None

    def __post_init__(self):
        if len(self.indices) == 0:
            raise ArgumentError("Must have at least one child index")


@dataclass
class MultiLevelIndex(AbstractANNIndex):
    """``MultiLevelIndex(root, merge_strategy, distance)`` (multilevel.jl:44-56)."""
    root: TransformedIndex
    merge_strategy: Any = field(default_factory=SimpleMerge)
    distance: Metric = default_distance
    _cache: dict = field(default_factory=dict, repr=False, compare=False)

    @property
    def dimension(self) -> int:
        return int(self.root.transform.centroids.shape[0])


def build_multilevel_index(X, config: TransformedConfig, *, merge_strategy=None, distance: Metric = default_distance,
                           seed: int = 0) -> MultiLevelIndex:
    """``build_index(MultiLevelIndex, X, config; merge_strategy=SimpleMerge(),
    distance)`` (builder.jl:61-80) for a KMeans transform over terminal
    children: fit a copy of the transform, partition the points by their
    final assignment (take_pending_assignments!, builder.jl:117-121), build
    one child per non-empty bucket (builder.jl:123-175)."""
    a = np.asarray(X)
    if a.ndim != 2:
        raise ArgumentError("X must be a d x n matrix")
    if not isinstance(config.transform, KMeansTransform):
        raise ArgumentError("the GPU MultiLevel builder takes a KMeansTransform")
    proto = config.transform
    t = KMeansTransform(k=proto.k, distance=proto.distance, init=proto.init, max_iters=proto.max_iters,
                        tol=proto.tol, subsample_size=proto.subsample_size)
    fit(t, a, seed=seed)
    assign = np.asarray(t.pending_assignments, np.int64)  # 1-based bucket of every point
    t.pending_assignments = None
    order = np.argsort(assign, kind="stable")
    counts = np.bincount(assign - 1, minlength=t.k)
    bucket_lookup = np.zeros(t.k, np.int64)
    id_mappings, children, pos = [], [], 0
    starts = np.concatenate([[0], np.cumsum(counts)])
    for b in range(t.k):
        if counts[b] == 0:
            continue
        ids = order[starts[b]:starts[b + 1]] + 1  # ascending parent ids, 1-based
        id_mappings.append(ids)
        child_cfg = config.child_config
        if child_cfg.index_type is not BruteForceIndex:
            raise ArgumentError("the GPU MultiLevel builder takes BruteForceIndex children")
        children.append(build_index(BruteForceIndex, a[:, ids - 1], distance=child_cfg.params.get(
            "distance", distance)))
        pos += 1
        bucket_lookup[b] = pos
    if not children:
        raise ArgumentError("Transform produced no non-empty buckets; cannot build child indices")
    root = TransformedIndex(t, config.routing, children, id_mappings, None, bucket_lookup)
    return MultiLevelIndex(root, merge_strategy or SimpleMerge(), distance)


# ---------------------------------------------------------------- routing
def _route(node: TransformedIndex, Qrows: np.ndarray) -> list:
    """Child positions (0-based) to probe for every query row: the transform's
    distances, select_indices of the routing strategy over the buckets,
    bucket -> child position (query.jl:305-345, _resolve_child_positions)."""
    t = node.transform
    D = pairwise_distances(np.ascontiguousarray(Qrows.T), t.centroids, t.distance)  # [nlist][nq]
    nb = t.k if node.bucket_lookup is not None else len(node.indices)
    pol = node.routing_strategy
    if isinstance(pol, TopKRouting):
        m = min(pol.k, nb)
        keys = (_order_keys(np.ascontiguousarray(D[:nb].T)).astype(np.uint64) << np.uint64(32)) | \
            np.arange(nb, dtype=np.uint64)[None, :]
        part = np.partition(keys, m - 1, axis=1)[:, :m] if m < nb else keys
        buckets = (np.sort(part, axis=1) & np.uint64(0xFFFFFFFF)).astype(np.int64)  # 0-based
        per_q = [row for row in buckets]
    else:
        per_q = [np.asarray(select_indices(pol, D[:, i], nb), np.int64) - 1 for i in range(D.shape[1])]
    if node.bucket_lookup is None:
        return per_q
    out = []
    for b in per_q:
        c = node.bucket_lookup[b] - 1
        out.append(c[c >= 0])
    return out


# ---------------------------------------------------------------- queries
def _child_results_per_child(ml: MultiLevelIndex, Xrows: np.ndarray, Qrows: np.ndarray, probes: list, k: int):
    """The reference's inverted batch loop on the GPU: one mann_knn_device per
    probed child over its sub-batch.  Returns per-query lists of per-child
    result lists (probe order), ids 1-based global."""
    import torch

    node = ml.root
    nq, d = Qrows.shape
    lib = _lib.load()
    perm = np.concatenate(node.id_mappings) - 1
    offs = np.concatenate([[0], np.cumsum([len(m) for m in node.id_mappings])])
    dev = torch.device("cuda")
    Xp = torch.from_numpy(np.ascontiguousarray(Xrows[perm])).to(dev)
    Qd = torch.from_numpy(np.ascontiguousarray(Qrows)).to(dev)
    per_child = [[] for _ in node.indices]
    for qi, cs in enumerate(probes):
        for c in cs:
            per_child[c].append(qi)
    results = [[None] * len(cs) for cs in probes]
    slot = [{int(c): j for j, c in enumerate(cs)} for cs in probes]
    stream = torch.cuda.current_stream().cuda_stream
    for c, qs in enumerate(per_child):
        if not qs:
            continue
        child = node.indices[c]
        nc = int(offs[c + 1] - offs[c])
        kk = min(int(k), nc)
        qidx = torch.from_numpy(np.asarray(qs, np.int64)).to(dev)
        Qs = Qd.index_select(0, qidx).contiguous()
        ids = torch.empty((len(qs), kk), dtype=torch.int32, device=dev)
        dd = torch.empty((len(qs), kk), dtype=torch.float32, device=dev)
        p = _lib.params(metric_code(child.distance), kk, _lib.PREC_FP32)
        base_ptr = Xp.data_ptr() + int(offs[c]) * d * 4
        _lib.check(lib.mann_knn_device(p, base_ptr, nc, Qs.data_ptr(), len(qs), d, ids.data_ptr(), dd.data_ptr(),
                                       None, C.c_void_p(stream)))
        ih, dh = ids.cpu().numpy(), dd.cpu().numpy()
        gmap = node.id_mappings[c]
        for j, qi in enumerate(qs):
            results[qi][slot[qi][c]] = [Neighbor(int(gmap[i]), float(x)) for i, x in zip(ih[j], dh[j]) if i >= 0]
    return results


def _scan_all(ml: MultiLevelIndex, Xrows: np.ndarray, Qrows: np.ndarray, probes: list, k: int):
    """All probed children in one mann_ivf_scan_device launch (disjoint
    BruteForce partitions): per query the (distance, id)-merged top-k."""
    import torch

    node = ml.root
    nq, d = Qrows.shape
    lib = _lib.load()
    key = ("lists", id(node))
    if key not in ml._cache:
        offs = np.concatenate([[0], np.cumsum([len(m) for m in node.id_mappings])]).astype(np.int64)
        ids = (np.concatenate(node.id_mappings) - 1).astype(np.int32)
        ml._cache[key] = (offs, ids)
    offs, lids = ml._cache[key]
    npb = max(1, max((len(p) for p in probes), default=1))
    pr = np.full((nq, npb), -1, np.int32)
    for i, p in enumerate(probes):
        pr[i, :len(p)] = p
    dev = torch.device("cuda")
    t = {n: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for n, v in
         (("X", Xrows), ("Q", Qrows), ("offs", offs), ("ids", lids), ("pr", pr))}
    oi = torch.empty((nq, k), dtype=torch.int32, device=dev)
    od = torch.empty((nq, k), dtype=torch.float32, device=dev)
    p = _lib.params(metric_code(node.indices[0].distance), k, _lib.PREC_FP32)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.mann_ivf_scan_device(p, t["pr"].data_ptr(), npb, t["X"].data_ptr(), Xrows.shape[0], d,
                                        len(node.indices), t["offs"].data_ptr(), t["ids"].data_ptr(),
                                        t["Q"].data_ptr(), nq, oi.data_ptr(), od.data_ptr(), C.c_void_p(stream)))
    ih, dh = oi.cpu().numpy(), od.cpu().numpy()
    return [[Neighbor(int(i) + 1, float(x)) for i, x in zip(ih[r], dh[r]) if i >= 0] for r in range(nq)]


def multilevel_query(ml: MultiLevelIndex, data, q, k: int, *, engine: str = "per_child"):
    """``query(index::MultiLevelIndex, data, q, k)``: q a vector (query.jl:25-39)
    -> list of Neighbor; q a d x m matrix or a list of vectors (query.jl:279-300)
    -> list of lists.  The batch routes every query, searches each probed child
    once for all its queries and merges per query with the index's strategy."""
    a = np.asarray(data)
    if isinstance(q, (list, tuple)):
        if len(q) == 0:
            return []
        Q = np.stack([np.asarray(v) for v in q], axis=1)
        single = False
    else:
        Q = np.asarray(q)
        single = Q.ndim == 1
        if single:
            Q = Q.reshape(-1, 1)
    if Q.shape[0] != a.shape[0]:
        raise DimensionMismatch(f"Expected queries with {a.shape[0]} rows, got {Q.shape[0]}")
    if Q.shape[1] == 0:
        return []
    k = int(k)
    if k <= 0:
        return [] if single else [[] for _ in range(Q.shape[1])]
    Xrows = points_view(a)
    Qrows = points_view(Q)
    probes = _route(ml.root, Qrows)
    if engine == "scan":
        if not (isinstance(ml.merge_strategy, (DisjointMerge, SimpleMerge)) and ml.root.id_mappings is not None):
            raise ArgumentError("the scan engine needs disjoint bucketed children")
        merged = _scan_all(ml, Xrows, Qrows, probes, k)
    elif engine == "per_child":
        lists = _child_results_per_child(ml, Xrows, Qrows, probes, k)
        merged = [merge_results(ml.merge_strategy, r, k) for r in lists]
    else:
        raise ArgumentError(f"unknown engine {engine!r}")
    return merged[0] if single else merged
