"""LearnedProbeRouting: a routing strategy beside TopKRouting
(src/indices/multilevel/routing.jl:14-118) that ranks the inverted lists of an
IVFFlatIndex with a small BF16 MLP trained on the GPU.

The network maps a query (din) through two GELU layers (hidden1, hidden2) to
one score per list; with the distance prior on, the score of list c is
``MLP(q)_c - beta * ||q - c||^2`` (beta learned).  It is trained with softmax
cross-entropy against the lists that hold the query's exact nearest
neighbours, which the GPU's exact search computes for a separate set of
training queries.  Training and inference are the library's own kernels
(``mann_probe_*`` in ``include/mann.h``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .distances import SqEuclidean, metric_code
from .indices import BruteForceIndex, knn_arrays, points_view


class ProbeModel:
    """Device-resident probe network (an owned ``mann_probe*``)."""

    def __init__(self, din, nout, hidden=(512, 512), *, use_prior=True, centroids=None, batch=1024,
                 lr=1e-3, weight_decay=1e-4, beta_init=1.0, seed=0, params=None):
        self.dims = (int(din), int(hidden[0]), int(hidden[1]), int(nout))
        self.use_prior = bool(use_prior)
        self.p = _lib.ProbeParams(self.dims[0], self.dims[1], self.dims[2], self.dims[3], int(batch),
                                  int(self.use_prior), lr, 0.9, 0.999, 1e-8, weight_decay, beta_init,
                                  int(seed) & (2**64 - 1))
        lib = _lib.load()
        n = lib.mann_probe_param_count(self.p)
        if n <= 0:
            raise ArgumentError("probe layer widths must be positive")
        if params is None:
            params = np.empty(n, np.float32)
            _lib.check(lib.mann_probe_init(self.p, params.ctypes.data))
        params = np.ascontiguousarray(params, np.float32)
        if params.size != n:
            raise DimensionMismatch(f"expected {n} parameters, got {params.size}")
        cent = None
        if self.use_prior:
            if centroids is None:
                raise ArgumentError("the distance prior needs the centroids")
            cent = np.ascontiguousarray(centroids, np.float32)  # [nout][din]
            if cent.shape != (self.dims[3], self.dims[0]):
                raise DimensionMismatch("centroids must be [nout][din]")
        self._cent = cent
        h = C.c_void_p()
        _lib.check(lib.mann_probe_create(self.p, params.ctypes.data, cent.ctypes.data if cent is not None else None,
                                         C.byref(h)))
        self.handle = h
        self.n_params = int(n)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.load().mann_probe_destroy(h)
            except Exception:
                pass
            self.handle = None

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        _lib.check(_lib.load().mann_probe_get_params(self.handle, out.ctypes.data))
        return out

    def save(self, path) -> None:
        """Write the network (flat parameters, widths, settings, centroids of the prior) to an .npz file."""
        p = self.p
        np.savez(path, format=np.array("manifoldann-gb300/probe/1"), params=self.params(),
                 dims=np.array(self.dims, np.int64), use_prior=np.int64(self.use_prior),
                 centroids=self._cent if self._cent is not None else np.zeros((0, 0), np.float32),
                 hyper=np.array([p.batch, p.lr, p.weight_decay, p.beta_init], np.float64), seed=np.uint64(p.seed))

    @classmethod
    def load(cls, path):
        """Re-create a network written by ``save`` on the current device."""
        with np.load(path) as z:
            if str(z["format"]) != "manifoldann-gb300/probe/1":
                raise ArgumentError(f"not a probe file: {path}")
            din, h1, h2, nout = (int(v) for v in z["dims"])
            batch, lr, wd, beta_init = z["hyper"].tolist()
            prior = bool(int(z["use_prior"]))
            return cls(din, nout, (h1, h2), use_prior=prior, centroids=z["centroids"] if prior else None,
                       batch=int(batch), lr=lr, weight_decay=wd, beta_init=beta_init, seed=int(z["seed"]),
                       params=z["params"])

    def train(self, queries, labels, epochs: int) -> np.ndarray:
        """queries [n][din] float32, labels [n][L] int32 list ids (-1 = none)."""
        q = np.ascontiguousarray(queries, np.float32)
        lab = np.ascontiguousarray(labels, np.int32)
        if q.shape[1] != self.dims[0]:
            raise DimensionMismatch("query width does not match the model")
        loss = np.empty(int(epochs), np.float32)
        _lib.check(_lib.load().mann_probe_train(self.handle, q.ctypes.data, q.shape[0], lab.ctypes.data,
                                                lab.shape[1], int(epochs), loss.ctypes.data))
        return loss

    def grad(self, queries, labels):
        q = np.ascontiguousarray(queries, np.float32)
        lab = np.ascontiguousarray(labels, np.int32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float(0)
        _lib.check(_lib.load().mann_probe_grad(self.handle, q.ctypes.data, q.shape[0], lab.ctypes.data,
                                               lab.shape[1], g.ctypes.data, C.byref(loss)))
        return float(loss.value), g

    def scores(self, queries) -> np.ndarray:
        q = np.ascontiguousarray(queries, np.float32)
        out = np.empty((q.shape[0], self.dims[3]), np.float32)
        _lib.check(_lib.load().mann_probe_scores(self.handle, q.ctypes.data, q.shape[0], out.ctypes.data))
        return out

    def route_device(self, queries_dev, nprobe: int, probes_dev, coverage_dev=None, stream: int = 0):
        def ptr(t):
            return None if t is None else (t if isinstance(t, int) else t.data_ptr())

        _lib.check(_lib.load().mann_probe_route_device(self.handle, ptr(queries_dev), queries_dev.shape[0],
                                                       int(nprobe), ptr(probes_dev), ptr(coverage_dev),
                                                       stream))


def list_of_points(index) -> np.ndarray:
    """0-based list id of every point of an IVFFlatIndex."""
    owner = np.empty(int(index.list_offsets[-1]), np.int32)
    o = index.list_offsets
    for c in range(index.nlist):
        owner[index.list_ids[o[c]:o[c + 1]]] = c
    return owner


def neighbour_list_labels(index, data, train_queries, k: int = 10) -> np.ndarray:
    """Labels [n][k]: the lists holding each training query's exact k nearest
    neighbours (exact search on the GPU), data d x N, queries d x n."""
    bf = BruteForceIndex(index.dimension, int(np.asarray(data).shape[1]), index.distance)
    ids, _ = knn_arrays(bf, data, train_queries, k, precision="auto")
    owner = list_of_points(index)
    lab = np.where(ids >= 0, owner[np.maximum(ids, 0)], -1).astype(np.int32)
    return lab


@dataclass
class LearnedProbeRouting:
    """``LearnedProbeRouting(k, model)``: probe the k lists with the highest scores."""
    k: int
    model: ProbeModel

    def __post_init__(self):
        if self.k <= 0:
            raise ArgumentError("k must be positive")

    @classmethod
    def train(cls, index, data, train_queries, *, k: int = 10, label_k: int = 10, hidden=(512, 512),
              epochs: int = 10, batch: int = 1024, lr: float = 1e-3, weight_decay: float = 1e-4,
              use_prior: bool = True, beta_init: float = 1.0, seed: int = 0):
        """Train on the GPU for an IVFFlatIndex built on ``data`` (d x N) with
        separate training queries (d x n)."""
        TQ = np.asarray(train_queries)
        labels = neighbour_list_labels(index, data, TQ, label_k)
        cent = np.ascontiguousarray(index.centroids.T, np.float32)
        model = ProbeModel(index.dimension, index.nlist, hidden, use_prior=use_prior, centroids=cent,
                           batch=batch, lr=lr, weight_decay=weight_decay, beta_init=beta_init, seed=seed)
        loss = model.train(points_view(TQ), labels, epochs)
        r = cls(k, model)
        r.loss_curve = loss
        return r

    def select(self, queries, nprobe: int | None = None) -> np.ndarray:
        """Probes [q][nprobe] (0-based list ids, best first) of queries d x q."""
        import torch

        Q = np.asarray(queries)
        if Q.ndim == 1:
            Q = Q.reshape(-1, 1)
        nprobe = self.k if nprobe is None else int(nprobe)
        nprobe = min(nprobe, self.model.dims[3])
        qd = torch.from_numpy(points_view(Q)).cuda()
        out = torch.empty((qd.shape[0], nprobe), dtype=torch.int32, device=qd.device)
        self.model.route_device(qd, nprobe, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()


def select_indices_learned(policy: LearnedProbeRouting, query, indices):
    """``select_indices`` for LearnedProbeRouting: 1-based list ids of the
    min(k, children) best-scored lists for one query vector."""
    n_children = indices if isinstance(indices, int) else len(indices)
    if n_children <= 0:
        return []
    m = min(policy.k, n_children, policy.model.dims[3])
    return (policy.select(np.asarray(query, np.float32), m)[0] + 1).tolist()


def ivf_search_learned(index, routing: LearnedProbeRouting, data, queries, k: int, nprobe: int | None = None):
    """IVF search routed by the probe: (ids [q][k] 0-based, dists [q][k])."""
    a = np.asarray(data)
    Q = np.asarray(queries)
    if Q.ndim == 1:
        Q = Q.reshape(-1, 1)
    index._check(a, Q.shape[0])
    nq = Q.shape[1]
    k = int(k)
    if k <= 0 or nq == 0:
        return np.empty((nq, 0), np.int32), np.empty((nq, 0), np.float32)
    nprobe = routing.k if nprobe is None else int(nprobe)
    X = points_view(a)
    qs = points_view(Q)
    ids = np.empty((nq, k), np.int32)
    dists = np.empty((nq, k), np.float32)
    p = _lib.params(metric_code(index.distance), k, _lib.PREC_FP32, 0, 0)
    _lib.check(_lib.load().mann_ivf_search_learned(
        routing.model.handle, p, nprobe, X.ctypes.data, X.shape[0], index.dimension, index.nlist,
        index.list_offsets.ctypes.data, index.list_ids.ctypes.data, qs.ctypes.data, nq, ids.ctypes.data,
        dists.ctypes.data))
    return ids, dists
