"""Full-size parity with the oracle on sampled rows.

The searches run at the full sizes of the measured workloads -- the 784-d
quantised mixture (60,000 points, 10,000 held-out queries and the 60,000-row
self graph), the 256-d angular set (290,000 points, 10,000 queries, cosine,
k = 20) and the 128-d anisotropic set (1,000,000 points, 10,000 queries) --
and a seeded sample of their result rows is checked against the CPU oracle:

* BF16 form: ids identical and distance bits identical to the FP32 oracle
  (the reference's BruteForceIndex semantics, src/indices/bruteforce.jl:46-71);
* BF16 form with MANN_FLAG_FP64_TIES: ids identical to the FP64 oracle, no
  unsettled row, and the reported max |distance - FP64 distance| equal to the
  one recomputed here on the sample (within its own rounding) and below the
  FP32 bound (d + 2) u |distance|.

The oracle rows are computed on every host core; the sample sizes keep each
test within seconds there.
"""
import numpy as np
import pytest

from test_knn_gpu import M_COS, M_SQ, gpu_graph, gpu_knn, same_bits

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def _rows(n, m, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(n, m), replace=False)).astype(np.int32)


def _err_bound(d, dists):
    # FP32 sequential difference-form sum: |fl(s) - s| <= (d + 2) u s (plus the
    # sqrt rounding for Euclidean), far below this for the tested metrics
    return 2.0 * (d + 2) * U * float(np.abs(dists).max()) + 1e-12


def _check_query_rows(orc, base, q, rows, k, metric, ids, dists, ids64, d64_rep, metric_o):
    ids_o, d_o = orc.knn_f32(base, q[rows], k, metric_o)
    assert np.array_equal(ids[rows], ids_o)
    assert same_bits(dists[rows], d_o)
    ids_o64, d_o64 = orc.knn_f64(base, q[rows], k, metric_o)
    assert np.array_equal(ids64[rows], ids_o64)
    return d_o64


def test_mixture_784_queries_and_graph_vs_oracle(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(60000, 784, seed=1)
    q = synthetic.quantized_mixture(10000, 784, seed=2)
    k = 10
    ids, dists, rep = gpu_knn(base, q, k, M_SQ, precision="bf16", report=True)
    ids64, d64, rep64 = gpu_knn(base, q, k, M_SQ, precision="bf16", fp64_ties=True, fp64_error=True,
                                report=True)
    assert rep["precision_used"] == 1 and rep64["precision_used"] == 1
    assert rep64["rows_unresolved"] == 0, rep64
    rows = _rows(10000, 1000, 11)
    d_o64 = _check_query_rows(orc, base, q, rows, k, M_SQ, ids, dists, ids64, rep64, orc.SQEUCLIDEAN)
    err_sample = float(np.abs(d64[rows].astype(np.float64) - d_o64).max())
    assert err_sample <= rep64["max_abs_err_fp64"] + 1e-12
    assert rep64["max_abs_err_fp64"] <= _err_bound(784, d64)
    # the self graph (build_knn_graph semantics), sampled rows
    g, gd, grep = gpu_graph(base, k, M_SQ, precision="bf16", report=True)
    g64, gd64, grep64 = gpu_graph(base, k, M_SQ, precision="bf16", fp64_ties=True, fp64_error=True,
                                  report=True)
    assert grep64["rows_unresolved"] == 0, grep64
    grows = _rows(60000, 1000, 12)
    go, gdo = orc.knn_graph_rows(base, grows, k, orc.SQEUCLIDEAN)
    assert np.array_equal(g[grows], go) and same_bits(gd[grows], gdo)
    go64, gdo64 = orc.knn_graph_rows(base, grows, k, orc.SQEUCLIDEAN, fp64=True)
    assert np.array_equal(g64[grows], go64)
    assert float(np.abs(gd64[grows].astype(np.float64) - gdo64).max()) <= grep64["max_abs_err_fp64"] + 1e-12
    assert grep64["max_abs_err_fp64"] <= _err_bound(784, gd64)


def test_angular_256_cosine_vs_oracle(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    base = synthetic.angular_clusters(290000, 256, seed=1)
    q = synthetic.angular_clusters(10000, 256, seed=2)
    k = 20
    ids, dists, rep = gpu_knn(base, q, k, M_COS, precision="bf16", report=True)
    ids64, d64, rep64 = gpu_knn(base, q, k, M_COS, precision="bf16", fp64_ties=True, fp64_error=True,
                                report=True)
    assert rep64["rows_unresolved"] == 0, rep64
    rows = _rows(10000, 400, 13)
    d_o64 = _check_query_rows(orc, base, q, rows, k, M_COS, ids, dists, ids64, rep64, orc.COSINE)
    assert float(np.abs(d64[rows].astype(np.float64) - d_o64).max()) <= rep64["max_abs_err_fp64"] + 1e-12
    # cosine distances carry an absolute error of order (d + 4) u
    assert rep64["max_abs_err_fp64"] <= 4.0 * (256 + 4) * U


def test_anisotropic_1m_128_vs_oracle(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    base = synthetic.anisotropic_clusters(1_000_000, 128, seed=1)
    q = synthetic.anisotropic_clusters(10000, 128, seed=3)
    k = 10
    ids, dists, rep = gpu_knn(base, q, k, M_SQ, precision="bf16", report=True)
    ids64, d64, rep64 = gpu_knn(base, q, k, M_SQ, precision="bf16", fp64_ties=True, fp64_error=True,
                                report=True)
    assert rep64["rows_unresolved"] == 0, rep64
    rows = _rows(10000, 300, 14)
    d_o64 = _check_query_rows(orc, base, q, rows, k, M_SQ, ids, dists, ids64, rep64, orc.SQEUCLIDEAN)
    assert float(np.abs(d64[rows].astype(np.float64) - d_o64).max()) <= rep64["max_abs_err_fp64"] + 1e-12
    assert rep64["max_abs_err_fp64"] <= _err_bound(128, d64)


def test_fp64_ties_widen_long_tie_clusters(gpu_lib, orc):
    """A tie at the k-th distance longer than the candidate list: 60 copies of
    each of 50 points, every query exactly on a point, so 60 candidates tie at
    distance 0 and the next cluster sits far away; plus 40 points equidistant
    from the query (a 40-long cluster at the k-th distance).  The rows are
    widened to their exact top-256 and still equal the FP64 oracle's order."""
    rng = np.random.default_rng(8)
    pts = rng.standard_normal((50, 64)).astype(np.float32)
    base = np.repeat(pts, 60, axis=0)
    q = pts[::7].copy()
    for precision in ("fp32", "bf16"):
        ids64, _, rep = gpu_knn(base, q, 10, M_SQ, precision=precision, fp64_ties=True, report=True)
        ids_o, _ = orc.knn_f64(base, q, 10, orc.SQEUCLIDEAN)
        assert np.array_equal(ids64, ids_o), precision
        assert rep["rows_unresolved"] == 0, rep
    # equidistant shell: 40 signed unit vectors e_i and -e_i scaled to radius 2
    # around the origin query, plus 12 closer points
    d = 32
    shell = np.concatenate([2.0 * np.eye(d, dtype=np.float32), -2.0 * np.eye(d, dtype=np.float32)])[:40]
    inner = (rng.standard_normal((12, d)) * 0.1).astype(np.float32)
    far = (rng.standard_normal((3000, d)) * 0.2 + 8.0).astype(np.float32)
    base2 = np.concatenate([far, shell, inner])
    q2 = np.zeros((3, d), np.float32)
    for precision in ("fp32", "bf16"):
        ids64, _, rep = gpu_knn(base2, q2, 20, M_SQ, precision=precision, fp64_ties=True, report=True)
        ids_o, _ = orc.knn_f64(base2, q2, 20, orc.SQEUCLIDEAN)
        assert np.array_equal(ids64, ids_o), precision
        assert rep["rows_unresolved"] == 0, rep
