"""Python binding of the CPU oracle (``oracle/liboracle.so``).

TEST INFRASTRUCTURE: imported only by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of bench.py, always as the checker or the timed CPU
baseline -- never by the ``manifoldann_gb300`` package.

Arrays follow the C ABI: points and queries row-major [n][d] float32, ids
0-based int32, short rows padded with -1 / +inf.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

EUCLIDEAN, SQEUCLIDEAN, COSINE = 0, 1, 2

_P, _I64, _I32 = C.c_void_p, C.c_int64, C.c_int32
_SIGS = {
    "orc_dist_f32": (C.c_float, [_P, _P, _I32, _I32]),
    "orc_dist_f64": (C.c_double, [_P, _P, _I32, _I32]),
    "orc_knn_f32": (_I32, [_P, _I64, _P, _I64, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_knn_f64": (_I32, [_P, _I64, _P, _I64, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_knn_graph_f32": (_I32, [_P, _I64, _I32, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_knn_graph_f64": (_I32, [_P, _I64, _I32, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_knn_graph_rows_f32": (_I32, [_P, _I64, _I32, _I32, _I32, _I32, _P, _I64, _P, _P, _I32]),
    "orc_knn_graph_rows_f64": (_I32, [_P, _I64, _I32, _I32, _I32, _I32, _P, _I64, _P, _P, _I32]),
    "orc_kmeans_assign_gemm_f32": (_I32, [_P, _I64, _P, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_kmeans_assign_f64": (_I32, [_P, _I64, _P, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_topk_route": (_I32, [_P, _I32, _I32, _I32, _P]),
    "orc_ivf_query_f32": (_I32, [_P, _I32, _P, _P, _I32, _P, _P, _P, _I64, _I32, _I32, _I32, _I32,
                                 _P, _P, _I32]),
    "orc_ivf_route_gemv_f32": (_I32, [_P, _P, _I32, _I32, _P, _I64, _I32, _I32, _P, _I32]),
    "cpu_bruteforce_batch": (_I32, [_P, _I64, _P, _I64, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_kmeanspp": (_I32, [_P, _I64, _I32, _I32, _I64, _P, _P]),
    "orc_kmeans_lloyd": (_I32, [_P, _I64, _I32, _I32, _P, _I32, C.c_double, _I32, _P, _P, _I32]),
    "orc_ivf_scan_f32": (_I32, [_P, _I32, _P, _P, _P, _I64, _P, _I32, _I32, _I32, _P, _P, _I32]),
    "orc_max_threads": (_I32, []),
}

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _check(rc):
    if rc != 0:
        raise ValueError(f"oracle returned status {rc} (ArgumentError)")


def dist_f32(x, y, metric):
    x, y = _f32(x), _f32(y)
    return float(load().orc_dist_f32(x.ctypes.data, y.ctypes.data, x.size, metric))


def dist_f64(x, y, metric):
    x, y = _f32(x), _f32(y)
    return float(load().orc_dist_f64(x.ctypes.data, y.ctypes.data, x.size, metric))


def knn_f32(base, queries, k, metric, threads=0):
    base, queries = _f32(base), _f32(queries)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    d = np.empty((nq, k), np.float32)
    _check(load().orc_knn_f32(base.ctypes.data, base.shape[0], queries.ctypes.data, nq,
                              base.shape[1], k, metric, ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def knn_f64(base, queries, k, metric, threads=0):
    base, queries = _f32(base), _f32(queries)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    d = np.empty((nq, k), np.float64)
    _check(load().orc_knn_f64(base.ctypes.data, base.shape[0], queries.ctypes.data, nq,
                              base.shape[1], k, metric, ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def knn_graph_f32(data, k, metric, include_self=False, threads=0):
    data = _f32(data)
    n = data.shape[0]
    ids = np.empty((n, k), np.int32)
    d = np.empty((n, k), np.float32)
    _check(load().orc_knn_graph_f32(data.ctypes.data, n, data.shape[1], k, int(include_self), metric,
                                    ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def knn_graph_f64(data, k, metric, include_self=False, threads=0):
    data = _f32(data)
    n = data.shape[0]
    ids = np.empty((n, k), np.int32)
    d = np.empty((n, k), np.float64)
    _check(load().orc_knn_graph_f64(data.ctypes.data, n, data.shape[1], k, int(include_self), metric,
                                    ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def knn_graph_rows(data, rows, k, metric, include_self=False, fp64=False, threads=0):
    """Rows `rows` of the kNN graph of `data` (row i of the result = point
    rows[i]), with the same semantics as knn_graph_f32 / knn_graph_f64."""
    data = _f32(data)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    ids = np.empty((len(rows), k), np.int32)
    d = np.empty((len(rows), k), np.float64 if fp64 else np.float32)
    fn = load().orc_knn_graph_rows_f64 if fp64 else load().orc_knn_graph_rows_f32
    _check(fn(data.ctypes.data, data.shape[0], data.shape[1], k, int(include_self), metric,
              rows.ctypes.data, len(rows), ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def kmeans_assign_gemm_f32(X, C_, metric, threads=0):
    X, C_ = _f32(X), _f32(C_)
    n = X.shape[0]
    a = np.empty(n, np.int32)
    d = np.empty(n, np.float32)
    _check(load().orc_kmeans_assign_gemm_f32(X.ctypes.data, n, C_.ctypes.data, C_.shape[0], X.shape[1],
                                             metric, a.ctypes.data, d.ctypes.data, threads))
    return a, d


def kmeans_assign_f64(X, C_, metric, threads=0):
    X, C_ = _f32(X), _f32(C_)
    n = X.shape[0]
    a = np.empty(n, np.int32)
    d = np.empty(n, np.float64)
    _check(load().orc_kmeans_assign_f64(X.ctypes.data, n, C_.ctypes.data, C_.shape[0], X.shape[1],
                                        metric, a.ctypes.data, d.ctypes.data, threads))
    return a, d


def topk_route(dists, n_children, k):
    dists = _f32(dists)
    out = np.empty(max(k, 1), np.int32)
    c = load().orc_topk_route(dists.ctypes.data, dists.size, n_children, k, out.ctypes.data)
    if c == -2:
        raise ValueError("Transform produced no routing distances for TopKRouting")
    return out[:c].copy()


def ivf_query_f32(data, centroids, centroid_norms, list_offsets, list_ids, queries, k, nprobe,
                  metric, centroid_metric, threads=0):
    data, centroids, centroid_norms, queries = map(_f32, (data, centroids, centroid_norms, queries))
    list_offsets = np.ascontiguousarray(list_offsets, dtype=np.int64)
    list_ids = np.ascontiguousarray(list_ids, dtype=np.int32)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    d = np.empty((nq, k), np.float32)
    _check(load().orc_ivf_query_f32(data.ctypes.data, data.shape[1], centroids.ctypes.data,
                                    centroid_norms.ctypes.data, centroids.shape[0],
                                    list_offsets.ctypes.data, list_ids.ctypes.data, queries.ctypes.data,
                                    nq, k, nprobe, metric, centroid_metric, ids.ctypes.data,
                                    d.ctypes.data, threads))
    return ids, d


def ivf_route_gemv_f32(centroids, centroid_norms, queries, nprobe, centroid_metric, threads=0):
    """Probes [nq][min(nprobe, nlist)] of the reference's IVF routing (GEMV-form
    centroid distances, then partialsortperm)."""
    centroids, centroid_norms, queries = map(_f32, (centroids, centroid_norms, queries))
    nlist = centroids.shape[0]
    np_ = max(1, min(int(nprobe), nlist))
    out = np.empty((queries.shape[0], np_), np.int32)
    _check(load().orc_ivf_route_gemv_f32(centroids.ctypes.data, centroid_norms.ctypes.data, nlist,
                                         centroids.shape[1], queries.ctypes.data, queries.shape[0], np_,
                                         centroid_metric, out.ctypes.data, threads))
    return out


def centroid_norms_f32(centroids):
    """||c||^2 of every centroid row as a sequential FP32 sum of squares (the
    reference's vec(sum(abs2, centroids; dims=1)), src/indices/ivf_flat.jl:82)."""
    c = _f32(centroids)
    out = np.zeros(c.shape[0], np.float32)
    for i in range(c.shape[1]):
        out = (out + c[:, i] * c[:, i]).astype(np.float32)
    return out


def ivf_scan_f32(data, list_offsets, list_ids, queries, probes, k, metric, threads=0):
    data, queries = _f32(data), _f32(queries)
    list_offsets = np.ascontiguousarray(list_offsets, dtype=np.int64)
    list_ids = np.ascontiguousarray(list_ids, dtype=np.int32)
    probes = np.ascontiguousarray(probes, dtype=np.int32)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    d = np.empty((nq, k), np.float32)
    _check(load().orc_ivf_scan_f32(data.ctypes.data, data.shape[1], list_offsets.ctypes.data,
                                   list_ids.ctypes.data, queries.ctypes.data, nq, probes.ctypes.data,
                                   probes.shape[1], k, metric, ids.ctypes.data, d.ctypes.data, threads))
    return ids, d


def cpu_bruteforce_batch(base, queries, k, metric, threads=0):
    base, queries = _f32(base), _f32(queries)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    d = np.empty((nq, k), np.float32)
    _check(load().cpu_bruteforce_batch(base.ctypes.data, base.shape[0], queries.ctypes.data, nq,
                                       base.shape[1], k, metric, ids.ctypes.data, d.ctypes.data,
                                       threads))
    return ids, d


def kmeanspp(X, k, first, u):
    X = _f32(X)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(k, np.int64)
    _check(load().orc_kmeanspp(X.ctypes.data, X.shape[0], X.shape[1], k, int(first), u.ctypes.data,
                               out.ctypes.data))
    return out


def kmeans_lloyd(X, C0, max_iters, tol, metric, threads=0):
    X = _f32(X)
    C_ = np.array(C0, dtype=np.float32, copy=True, order="C")
    a = np.empty(X.shape[0], np.int32)
    it = np.zeros(1, np.int32)
    _check(load().orc_kmeans_lloyd(X.ctypes.data, X.shape[0], X.shape[1], C_.shape[0], C_.ctypes.data,
                                   max_iters, tol, metric, a.ctypes.data, it.ctypes.data, threads))
    return C_, a, int(it[0])


def max_threads() -> int:
    return int(load().orc_max_threads())
