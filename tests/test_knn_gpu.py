"""Parity of the FP32 fused top-k kernel (MANN_PREC_FP32) with the oracle:
ids identical and distances bit-identical (the kernel reproduces the oracle's
sequential fused multiply-add sum), on the reference's known answers, the
golden fixtures and seeded inputs of the plain-kNN workload."""
import threading

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

M_EUC, M_SQ, M_COS = 0, 1, 2


def gpu_knn(base, q, k, metric, precision="fp32", **kw):
    import manifoldann_gb300 as M

    metric_obj = {M_EUC: M.Euclidean(), M_SQ: M.SqEuclidean(), M_COS: M.CosineDist()}[metric]
    index = M.build_index(M.BruteForceIndex, base.T, distance=metric_obj)
    return M.knn_arrays(index, base.T, q.T, k, precision=precision, **kw)


def gpu_graph(data, k, metric, include_self=False, precision="fp32", **kw):
    import manifoldann_gb300 as M

    metric_obj = {M_EUC: M.Euclidean(), M_SQ: M.SqEuclidean(), M_COS: M.CosineDist()}[metric]
    index = M.build_index(M.BruteForceIndex, data.T, distance=metric_obj)
    return M.knn_graph_arrays(index, data.T, k, include_self=include_self, precision=precision, **kw)


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def test_known_answer_bruteforce(gpu_lib):
    import manifoldann_gb300 as M

    data = np.array([[0.0, 1.0, 2.0], [0.0, 0.0, 0.0]])
    index = M.build_index(M.BruteForceIndex, data)
    nb = M.query(index, data, np.array([0.25, 0.0]), 2)
    assert M.neighbor_ids(nb) == [1, 2]
    assert nb[0].dist == pytest.approx(0.25) and nb[1].dist == pytest.approx(0.75)


def test_default_distance_helpers(gpu_lib):
    import manifoldann_gb300 as M

    x = np.array([1.0, 2.0, 3.0], np.float32)
    y = np.array([1.5, 2.5, -1.0], np.float32)
    d = M.default_distance(x, y)
    dsq = M.default_squared_distance(x, y)
    assert d >= 0 and dsq >= 0 and abs(np.float32(d) ** 2 - dsq) <= 1e-5


def test_known_answer_graph_collinear(gpu_lib):
    import manifoldann_gb300 as M

    data = np.arange(1, 13, dtype=np.float64).reshape(4, 3).T  # reshape(1:12, 3, 4)
    index = M.build_index(M.BruteForceIndex, data)
    g = M.build_knn_graph(index, data, k=2)
    assert g.k == 2 and g.include_self is False and len(g) == 4
    assert g.neighbors == [[2, 3], [1, 3], [2, 4], [3, 2]]  # ties -> lower id
    gs = M.build_knn_graph(index, data, k=3, include_self=True)
    for i, nb in enumerate(gs.neighbors):
        assert len(nb) == 3 and (i + 1) in nb
    gm = M.build_knn_graph(index, data, k=2, metadata=[f"p{i}" for i in range(1, 5)])
    assert M.has_metadata(gm) and M.node_metadata(gm, 3) == "p3"
    gu = M.build_knn_graph(index, data, k=1, directed=False)
    assert gu.metadata["original_k"] == 1 and gu.k == max(len(n) for n in gu.neighbors)


@pytest.mark.parametrize("name", ["knn_iid_sq_d64", "knn_iid_euclid_d64", "knn_iid_cos_d37",
                                  "knn_mix_sq_d784", "knn_ang_cos_d256"])
def test_fp32_matches_golden(gpu_lib, name):
    g = load_golden(name)
    ids, d = gpu_knn(g["base"], g["queries"], int(g["k"]), int(g["metric"]))
    assert np.array_equal(ids, g["ids_f32"])
    assert same_bits(d, g["dists_f32"])


@pytest.mark.parametrize("name", ["graph_mix_sq_d784", "graph_cloud_sq_d32", "graph_cloud_sq_d32_self"])
def test_fp32_graph_matches_golden(gpu_lib, name):
    g = load_golden(name)
    ids, d = gpu_graph(g["data"], int(g["k"]), int(g["metric"]), bool(g["include_self"]))
    assert np.array_equal(ids, g["ids_f32"])
    assert same_bits(d, g["dists_f32"])


def test_fp32_plain_workload_full_size(gpu_lib, orc):
    # N=10,000 points, Q=1,000 queries, d=64, N(0,1), SqEuclidean, k=10
    from manifoldann_gb300 import synthetic

    base = synthetic.iid_normal(10000, 64, seed=1)
    q = synthetic.iid_normal(1000, 64, seed=2)
    ids, d = gpu_knn(base, q, 10, M_SQ)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o)
    assert same_bits(d, d_o)
    rel = np.abs(d - d_o) / np.maximum(np.abs(d_o), 1e-30)
    assert rel.max() <= 1e-5


@pytest.mark.parametrize("k", [1, 7, 32, 33, 64, 65, 128, 200, 256])
def test_fp32_k_range(gpu_lib, orc, k):
    rng = np.random.default_rng(k)
    base = rng.standard_normal((3001, 24)).astype(np.float32)
    q = rng.standard_normal((150, 24)).astype(np.float32)
    ids, d = gpu_knn(base, q, k, M_SQ)
    ids_o, d_o = orc.knn_f32(base, q, k, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o) and same_bits(d, d_o)


@pytest.mark.parametrize("n,d,k", [(1, 5, 3), (5, 1, 10), (129, 3, 200), (64, 4, 64), (300, 130, 11)])
def test_fp32_edge_shapes(gpu_lib, orc, n, d, k):
    rng = np.random.default_rng(n * 1000 + d)
    base = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((7, d)).astype(np.float32)
    ids, dist = gpu_knn(base, q, k, M_EUC)
    ids_o, d_o = orc.knn_f32(base, q, min(k, n), orc.EUCLIDEAN)
    assert ids.shape == (7, min(k, n))
    assert np.array_equal(ids, ids_o) and same_bits(dist, d_o)


@pytest.mark.parametrize("nq,n,d,k,metric", [(1, 60000, 784, 10, M_SQ), (3, 20000, 129, 40, M_EUC), (4, 9000, 2048, 7, M_COS),
                                              (2, 5000, 37, 64, M_SQ), (5, 7000, 64, 12, M_SQ), (4, 3000, 2100, 5, M_EUC)])
def test_fp32_few_rows_equal_oracle(gpu_lib, orc, nq, n, d, k, metric):
    """A handful of query rows (the shared-memory staged scan for <= 4 rows of
    d <= 2048, the chunked one above): ids and distance bits of the oracle."""
    rng = np.random.default_rng(nq * 1000 + d)
    base = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((nq, d)).astype(np.float32)
    ids, dd = gpu_knn(base, q, k, metric)
    ids_o, d_o = orc.knn_f32(base, q, k, metric)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dd, d_o)


def test_fp32_exact_ties_and_duplicates(gpu_lib, orc):
    # all-equal points: every distance ties, the order must be by id
    base = np.ones((500, 8), np.float32)
    base[250:] = 2.0
    q = np.ones((3, 8), np.float32)
    ids, _ = gpu_knn(base, q, 40, M_SQ)
    assert ids.tolist() == [list(range(40))] * 3
    # integer lattice points: many exact ties
    rng = np.random.default_rng(7)
    base = rng.integers(0, 3, size=(4000, 6)).astype(np.float32)
    q = rng.integers(0, 3, size=(100, 6)).astype(np.float32)
    ids, d = gpu_knn(base, q, 50, M_SQ)
    ids_o, d_o = orc.knn_f32(base, q, 50, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o) and same_bits(d, d_o)


def test_fp32_nan_sorts_last(gpu_lib):
    base = np.array([[np.nan, 0.0], [1.0, 0.0], [0.5, 0.0]], np.float32)
    ids, d = gpu_knn(base, np.zeros((1, 2), np.float32), 3, M_SQ)
    assert ids[0].tolist() == [2, 1, 0] and np.isnan(d[0, 2])


def test_cosine_zero_norm_is_nan_last(gpu_lib, orc):
    base = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]], np.float32)
    q = np.array([[1.0, 0.2]], np.float32)
    ids, d = gpu_knn(base, q, 3, M_COS)
    ids_o, d_o = orc.knn_f32(base, q, 3, orc.COSINE)
    assert ids.tolist() == ids_o.tolist() and np.isnan(d[0, 2])


def test_batch_equals_single_queries(gpu_lib):
    # test/unit/indices/abstract_batch_query_tests.jl:19-60 (batch == per-query loop)
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0xBA7CE5)
    data = rng.standard_normal((16, 1000)).astype(np.float32)
    Q = rng.standard_normal((16, 80)).astype(np.float32)
    index = M.build_index(M.BruteForceIndex, data)
    batch = M.query(index, data, Q, 5)
    single = [M.query(index, data, Q[:, i], 5) for i in range(80)]
    assert batch == single
    vecs = M.query(index, data, [Q[:, i] for i in range(80)], 5)
    assert vecs == batch


def test_device_pointer_entry_points(gpu_lib, orc):
    import ctypes as C

    import torch

    from manifoldann_gb300 import _lib

    rng = np.random.default_rng(3)
    base = rng.standard_normal((5000, 32)).astype(np.float32)
    q = rng.standard_normal((300, 32)).astype(np.float32)
    tb, tq = torch.from_numpy(base).cuda(), torch.from_numpy(q).cuda()
    ids = torch.empty((300, 10), dtype=torch.int32, device="cuda")
    d = torch.empty((300, 10), dtype=torch.float32, device="cuda")
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, 10)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(gpu_lib.mann_knn_device(p, tb.data_ptr(), 5000, tq.data_ptr(), 300, 32, ids.data_ptr(),
                                       d.data_ptr(), None, C.c_void_p(stream)))
    torch.cuda.synchronize()
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    assert np.array_equal(ids.cpu().numpy(), ids_o) and same_bits(d.cpu().numpy(), d_o)
    gi = torch.empty((5000, 6), dtype=torch.int32, device="cuda")
    gd = torch.empty((5000, 6), dtype=torch.float32, device="cuda")
    p6 = _lib.params(_lib.METRIC_SQEUCLIDEAN, 6)
    _lib.check(gpu_lib.mann_knn_graph_device(p6, tb.data_ptr(), 5000, 32, 0, gi.data_ptr(), gd.data_ptr(),
                                             None, C.c_void_p(stream)))
    torch.cuda.synchronize()
    gi_o, gd_o = orc.knn_graph_f32(base, 6, orc.SQEUCLIDEAN)
    assert np.array_equal(gi.cpu().numpy(), gi_o) and same_bits(gd.cpu().numpy(), gd_o)


def test_concurrent_host_calls(gpu_lib, orc):
    # the re-entrancy contract of src/ann_index.jl:60-66: concurrent callers
    rng = np.random.default_rng(11)
    base = rng.standard_normal((4000, 48)).astype(np.float32)
    qs = [rng.standard_normal((64, 48)).astype(np.float32) for _ in range(8)]
    out = [None] * 8

    def work(i):
        out[i] = gpu_knn(base, qs[i], 9, M_SQ)

    th = [threading.Thread(target=work, args=(i,)) for i in range(8)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i in range(8):
        ids_o, d_o = orc.knn_f32(base, qs[i], 9, orc.SQEUCLIDEAN)
        assert np.array_equal(out[i][0], ids_o) and same_bits(out[i][1], d_o)
