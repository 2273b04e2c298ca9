"""The CPU oracle against the reference's own known answers and against an
exact-arithmetic restatement of its summation (no GPU needed)."""
from fractions import Fraction

import numpy as np
import pytest

from conftest import load_golden

# ---------------------------------------------------------------- known answers


def test_bruteforce_known_answer(orc):
    # test/unit/indices/bruteforce_tests.jl:22-27: data=[0 1 2; 0 0 0], q=[0.25, 0], k=2 -> [1, 2]
    data = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], np.float32)  # rows = points
    q = np.array([[0.25, 0.0]], np.float32)
    for metric in (orc.EUCLIDEAN, orc.SQEUCLIDEAN):
        ids, _ = orc.knn_f32(data, q, 2, metric)
        assert list(ids[0] + 1) == [1, 2]


def test_default_distance_helpers(orc):
    # test/unit/indices/bruteforce_tests.jl:4-13
    x = np.array([1.0, 2.0, 3.0], np.float32)
    y = np.array([1.5, 2.5, -1.0], np.float32)
    d = orc.dist_f32(x, y, orc.EUCLIDEAN)
    dsq = orc.dist_f32(x, y, orc.SQEUCLIDEAN)
    assert d >= 0 and dsq >= 0
    assert abs(np.float32(d) ** 2 - dsq) <= 1e-5


def collinear():
    # test/unit/graphs/graph_tests.jl:4-48: reshape(1:12, 3, 4) -> 4 equally spaced points
    return np.arange(1, 13, dtype=np.float32).reshape(4, 3)


def test_graph_collinear_ties(orc):
    data = collinear()
    ids, d = orc.knn_graph_f32(data, 2, orc.SQEUCLIDEAN, include_self=False)
    # middle points see two neighbours at the same distance: the lower id comes first
    assert (ids + 1).tolist() == [[2, 3], [1, 3], [2, 4], [3, 2]]
    for i, row in enumerate(ids):
        assert i not in row
    ids_s, _ = orc.knn_graph_f32(data, 3, orc.SQEUCLIDEAN, include_self=True)
    for i, row in enumerate(ids_s):
        assert len(row) == 3 and i in row
    with pytest.raises(ValueError):
        orc.knn_graph_f32(data, 0, orc.SQEUCLIDEAN)
    with pytest.raises(ValueError):
        orc.knn_graph_f32(data, 4, orc.SQEUCLIDEAN, include_self=False)


def test_topk_routing_known_answers(orc):
    # test/unit/indices/multilevel/routing_tests.jl:8-56
    d = np.array([0.9, 0.8, 0.7, 0.6, 0.5, 0.1, 0.2], np.float32)
    assert (orc.topk_route(d, 5, 3) + 1).tolist() == [5, 4, 3]
    d = np.array([0.4, 0.3, 0.2, 0.1], np.float32)
    assert (orc.topk_route(d, 4, 10) + 1).tolist() == [4, 3, 2, 1]
    assert orc.topk_route(np.array([0.1, 0.2], np.float32), 0, 3).tolist() == []
    with pytest.raises(ValueError):
        orc.topk_route(np.array([], np.float32), 3, 5)


def test_kmeans_self_distance_clamped(orc):
    # test/unit/transforms/test_kmeans_optimizations.jl:107-122
    rng = np.random.default_rng(0)
    X = rng.random((10, 100), dtype=np.float32)
    C = X[:5].copy()
    a, dist = orc.kmeans_assign_gemm_f32(X, C, orc.EUCLIDEAN)
    assert (a[:5] == np.arange(5)).all()
    assert (dist[:5] >= 0).all() and (dist[:5] <= 0.01).all()


def test_kmeans_assign_strict_lowest_id(orc):
    # assign_clusters! keeps the first minimum (strict <): duplicate centroids -> lowest id
    X = np.array([[0.0, 0.0], [5.0, 5.0]], np.float32)
    C = np.array([[1.0, 1.0], [1.0, 1.0], [5.0, 5.0], [5.0, 5.0]], np.float32)
    a, _ = orc.kmeans_assign_f64(X, C, orc.SQEUCLIDEAN)
    assert a.tolist() == [0, 2]
    a, _ = orc.kmeans_assign_gemm_f32(X, C, orc.SQEUCLIDEAN)
    assert a.tolist() == [0, 2]


# ------------------------------------------------- exact restatement, small cases


def _round_f32(x: Fraction) -> np.float32:
    """Correctly rounded (nearest, ties-to-even) float32 of an exact rational."""
    c = np.float32(float(x))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        err = abs(Fraction(float(cand)) - x)
        key = (err, int(np.frombuffer(np.float32(cand).tobytes(), np.uint32)[0]) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return np.float32(best[1])


def _exact_sq_f32(x, y):
    s = np.float32(0.0)
    for a, b in zip(x, y):
        t = np.float32(a) - np.float32(b)  # one rounding, as fl(x - y)
        s = _round_f32(Fraction(float(s)) + Fraction(float(t)) ** 2)  # fmaf(t, t, s)
    return s


def test_oracle_summation_is_sequential_fma(orc):
    rng = np.random.default_rng(5)
    for d in (1, 3, 8, 17):
        for _ in range(20):
            x = rng.standard_normal(d).astype(np.float32) * np.float32(rng.uniform(0.01, 100))
            y = rng.standard_normal(d).astype(np.float32)
            assert orc.dist_f32(x, y, orc.SQEUCLIDEAN) == _exact_sq_f32(x, y)


def test_oracle_f64_matches_numpy_order(orc):
    rng = np.random.default_rng(9)
    base = rng.standard_normal((300, 12)).astype(np.float32)
    q = rng.standard_normal((20, 12)).astype(np.float32)
    ids, d = orc.knn_f64(base, q, 7, orc.SQEUCLIDEAN)
    ref = ((q[:, None, :].astype(np.float64) - base[None, :, :]) ** 2).sum(-1)
    order = np.lexsort((np.broadcast_to(np.arange(300), ref.shape), ref), axis=1)[:, :7]
    assert (ids == order).all()
    assert np.allclose(d, np.take_along_axis(ref, order, 1), rtol=1e-12)


def test_oracle_pads_short_rows(orc):
    base = np.zeros((3, 4), np.float32)
    ids, d = orc.knn_f32(base, np.zeros((2, 4), np.float32), 5, orc.SQEUCLIDEAN)
    assert ids[:, :3].tolist() == [[0, 1, 2]] * 2 and (ids[:, 3:] == -1).all()
    assert np.isinf(d[:, 3:]).all()


def test_oracle_nan_sorts_last(orc):
    base = np.array([[np.nan, 0.0], [1.0, 0.0], [0.5, 0.0]], np.float32)
    ids, d = orc.knn_f32(base, np.zeros((1, 2), np.float32), 3, orc.SQEUCLIDEAN)
    assert ids[0].tolist() == [2, 1, 0] and np.isnan(d[0, 2])


@pytest.mark.parametrize("name", ["knn_iid_sq_d64", "knn_iid_euclid_d64", "knn_iid_cos_d37",
                                  "knn_mix_sq_d784", "knn_ang_cos_d256"])
def test_oracle_reproduces_golden(orc, name):
    g = load_golden(name)
    k, m = int(g["k"]), int(g["metric"])
    ids, d = orc.knn_f32(g["base"], g["queries"], k, m)
    assert (ids == g["ids_f32"]).all() and (d.view(np.uint32) == g["dists_f32"].view(np.uint32)).all()
    ids64, d64 = orc.knn_f64(g["base"], g["queries"], k, m)
    assert (ids64 == g["ids_f64"]).all() and (d64 == g["dists_f64"]).all()


@pytest.mark.parametrize("name", ["graph_mix_sq_d784", "graph_cloud_sq_d32", "graph_cloud_sq_d32_self"])
def test_oracle_graph_golden(orc, name):
    g = load_golden(name)
    ids, d = orc.knn_graph_f32(g["data"], int(g["k"]), int(g["metric"]), bool(g["include_self"]))
    assert (ids == g["ids_f32"]).all() and (d == g["dists_f32"]).all()


def test_graph_equals_knn_minus_self(orc):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((400, 16)).astype(np.float32)
    gi, _ = orc.knn_graph_f32(x, 8, orc.SQEUCLIDEAN)
    ki, _ = orc.knn_f32(x, x, 9, orc.SQEUCLIDEAN)
    for i in range(400):
        assert gi[i].tolist() == [j for j in ki[i] if j != i][:8]


def test_cpu_baseline_agrees(orc):
    rng = np.random.default_rng(4)
    base = rng.standard_normal((3000, 64)).astype(np.float32)
    q = rng.standard_normal((100, 64)).astype(np.float32)
    ids, d = orc.cpu_bruteforce_batch(base, q, 10, orc.SQEUCLIDEAN)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    assert (ids == ids_o).mean() > 0.99
    assert np.allclose(d, d_o, rtol=1e-5)


def test_ivf_oracle_full_probe_is_exact(orc):
    rng = np.random.default_rng(8)
    data = rng.standard_normal((500, 8)).astype(np.float32)
    cents = data[:10].copy()
    a, _ = orc.kmeans_assign_f64(data, cents, orc.SQEUCLIDEAN)
    order = np.argsort(a, kind="stable")
    offs = np.concatenate([[0], np.cumsum(np.bincount(a, minlength=10))])
    cn = (cents.astype(np.float64) ** 2).sum(1).astype(np.float32)
    q = rng.standard_normal((30, 8)).astype(np.float32)
    ids, d = orc.ivf_query_f32(data, cents, cn, offs, order.astype(np.int32), q, 5, 10,
                               orc.SQEUCLIDEAN, orc.SQEUCLIDEAN)
    ids_e, d_e = orc.knn_f32(data, q, 5, orc.SQEUCLIDEAN)
    assert (ids == ids_e).all() and (d == d_e).all()
