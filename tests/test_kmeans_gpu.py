"""KMeans on the GPU against the oracle: pairwise distances (bits), exact
assignment (ids), k-means++ with the same draws (indices), Lloyd from the
same initial centroids (centroid bits, assignments, iteration count), and the
reference's own KMeans tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rows(a):
    return np.ascontiguousarray(np.asarray(a, np.float32))


@pytest.mark.parametrize("metric", [0, 1, 2])
def test_pairwise_distances_bits(gpu_lib, orc, metric):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(metric)
    X = rng.standard_normal((333, 29)).astype(np.float32)
    C = rng.standard_normal((70, 29)).astype(np.float32)
    m = {0: M.Euclidean(), 1: M.SqEuclidean(), 2: M.CosineDist()}[metric]
    D = M.pairwise_distances(X.T, C.T, m)  # k x n
    assert D.shape == (70, 333)
    for j in range(0, 333, 37):
        for i in range(0, 70, 9):
            assert np.float32(D[i, j]).view(np.uint32) == np.float32(orc.dist_f32(X[j], C[i], metric)).view(np.uint32)


def test_negative_squared_distance_clamping(gpu_lib):
    # test/unit/transforms/test_kmeans_optimizations.jl:107-122
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0)
    X = rng.random((100, 10), dtype=np.float32)  # d x n
    C = X[:, :5].copy()
    D = M.pairwise_distances(X, C, M.Euclidean())
    for i in range(5):
        assert D[i, i] >= 0 and D[i, i] <= 0.01


@pytest.mark.parametrize("n,k,d,metric", [(5000, 64, 16, 1), (3000, 300, 128, 0), (20000, 4096, 128, 1)])
def test_assign_is_exact_argmin(gpu_lib, orc, n, k, d, metric):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, d)).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)] + 0.01 * rng.standard_normal((k, d)).astype(np.float32)
    a, dist = M.assign_arrays(X.T, C.T, M.Euclidean() if metric == 0 else M.SqEuclidean())
    a_o, d_o = orc.kmeans_assign_f64(X, C, metric)
    assert np.array_equal(a, a_o)
    assert np.allclose(dist, d_o, rtol=1e-5)


def test_assign_ties_to_lowest_centroid(gpu_lib):
    import manifoldann_gb300 as M

    X = np.array([[0.0, 0.0], [5.0, 5.0]], np.float32)
    C = np.array([[1.0, 1.0], [1.0, 1.0], [5.0, 5.0], [5.0, 5.0]], np.float32)
    assert M.assign_clusters(X.T, C.T, M.SqEuclidean()).tolist() == [1, 3]


def test_kmeanspp_same_draws_same_points(gpu_lib, orc):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(7)
    X = rng.standard_normal((9000, 24)).astype(np.float32)
    k = 40
    u = rng.random(k)
    C, idx = M.init_kmeans_plus_plus(X.T, k, first=123, u=u)
    idx_o = orc.kmeanspp(X, k, 122, u)
    assert np.array_equal(idx - 1, idx_o)
    assert len(set(idx.tolist())) == k
    assert np.array_equal(C, X[idx_o].T)


@pytest.mark.parametrize("metric", [0, 1])
def test_lloyd_matches_oracle_bits(gpu_lib, orc, metric):
    import manifoldann_gb300 as M

    from manifoldann_gb300 import synthetic

    X = synthetic.anisotropic_clusters(12000, 32, seed=2, clusters=50)
    rng = np.random.default_rng(3)
    C0 = X[rng.choice(len(X), 64, replace=False)]
    C, a, it = M.lloyd(C0.T, X.T, M.Euclidean() if metric == 0 else M.SqEuclidean(), max_iters=15,
                       tol=1e-4)
    C_o, a_o, it_o = orc.kmeans_lloyd(X, C0, 15, 1e-4, metric)
    assert it == it_o
    assert np.array_equal(a - 1, a_o)
    assert np.array_equal(C.T.view(np.uint32), C_o.view(np.uint32))


def test_lloyd_empty_clusters_get_distinct_points(gpu_lib, orc):
    # test/unit/transforms/test_kmeans_rng_and_empty_clusters.jl:7-51
    import manifoldann_gb300 as M

    X = np.array([[0.0, 1.0, 2.0, 3.0, 4.0], [0.0, 0.0, 0.0, 0.0, 0.0]], np.float32)  # d x n
    C0 = np.array([[0.0, 1e9, 1e9, 1e9], [0.0, 1e9, 1e9, 1e9]], np.float32)
    C, _, _ = M.lloyd(C0, X, M.Euclidean(), max_iters=1)
    rep = [tuple(C[:, i]) for i in range(1, 4)]
    assert len(set(rep)) == 3
    cols = [tuple(X[:, j]) for j in range(5)]
    assert all(r in cols for r in rep)
    C_o, _, _ = orc.kmeans_lloyd(X.T, C0.T, 1, 1e-6, 0)
    assert np.array_equal(C.T, C_o)


def test_fit_is_deterministic_and_consistent(gpu_lib, orc):
    import manifoldann_gb300 as M

    from manifoldann_gb300 import synthetic

    X = synthetic.anisotropic_clusters(20000, 32, seed=5, clusters=40).T  # d x n
    t1 = M.fit(M.KMeansTransform(k=40, distance=M.Euclidean(), max_iters=25, tol=1e-4), X, seed=11)
    t2 = M.fit(M.KMeansTransform(k=40, distance=M.Euclidean(), max_iters=25, tol=1e-4), X, seed=11)
    assert np.array_equal(t1.centroids, t2.centroids)
    a1 = M.take_pending_assignments(t1)
    assert t1.pending_assignments is None
    a_o, _ = orc.kmeans_assign_f64(X.T, t1.centroids.T, 0)
    assert np.array_equal(a1 - 1, a_o)
    # subsampled Lloyd + full assignment
    t3 = M.fit(M.KMeansTransform(k=40, distance=M.SqEuclidean(), init="random", max_iters=10,
                                 tol=1e-4, subsample_size=5000), X, seed=1)
    a3 = M.take_pending_assignments(t3)
    assert len(a3) == 20000 and a3.min() >= 1 and a3.max() <= 40
    r = M.transform(t3, X[:, 0])
    assert r.assignment.distances.shape == (40,)
    assert M.get_bucket_assignment(r.assignment) == a3[0]


def test_kmeans_transform_validation(gpu_lib):
    import manifoldann_gb300 as M

    with pytest.raises(M.ArgumentError):
        M.KMeansTransform(k=0, distance=M.Euclidean())
    with pytest.raises(M.ArgumentError):
        M.KMeansTransform(k=3, distance=M.Euclidean(), init="bogus")
    t = M.KMeansTransform(k=3, distance=M.Euclidean())
    with pytest.raises(M.ArgumentError):
        M.transform(t, np.zeros(4, np.float32))
    with pytest.raises(M.ArgumentError):
        M.fit(t, np.zeros((4, 2), np.float32))
