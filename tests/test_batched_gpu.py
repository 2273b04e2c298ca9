"""Batched kNN graphs of many uneven point sets in one persistent launch over
a device work queue (replayed from a captured CUDA graph): every set's graph
equals the oracle's build_knn_graph of that set alone (ids and distance bits,
k + 1 up to 64), at full size it equals the one-set GPU graph of each cloud,
and graph replays and re-plans give the same bytes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clouds(count, lo, hi, d, seed):
    from manifoldann_gb300 import synthetic

    return synthetic.manifold_clouds(count, lo, hi, d, seed=seed)


@pytest.mark.parametrize("metric,d,k,include_self", [(1, 32, 15, False), (0, 7, 5, True), (1, 12, 31, False),
                                                    (1, 32, 40, False), (0, 9, 64, True), (1, 32, 63, False)])
def test_batched_graphs_equal_oracle_per_set(gpu_lib, orc, metric, d, k, include_self):
    import manifoldann_gb300 as M

    clouds = _clouds(7, 200, 3000, d, seed=d)
    dist = M.SqEuclidean() if metric == 1 else M.Euclidean()
    ids, dists, offs, rep = M.knn_graph_batched_arrays([c.T for c in clouds], k, distance=dist,
                                                       include_self=include_self, report=True)
    assert rep["rows"] == offs[-1]
    for c, cl in enumerate(clouds):
        i_o, d_o = orc.knn_graph_f32(cl, k, metric, include_self=include_self)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i_o), c
        assert np.array_equal(dists[offs[c]:offs[c + 1]].view(np.uint32), d_o.view(np.uint32)), c


def test_batched_ties_and_duplicates(gpu_lib, orc):
    import manifoldann_gb300 as M

    g = np.stack(np.meshgrid(np.arange(6), np.arange(5), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    a = np.concatenate([g, g[:17]]).astype(np.float32)  # exact ties and duplicate points
    b = (np.arange(40, dtype=np.float32)[:, None] * np.ones((1, 3), np.float32))
    ids, dists, offs = M.knn_graph_batched_arrays([a.T, b.T], 6, distance=M.SqEuclidean())
    for c, cl in enumerate((a, b)):
        i_o, d_o = orc.knn_graph_f32(cl, 6, 1)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i_o)
        assert np.array_equal(dists[offs[c]:offs[c + 1]], d_o)
    graphs = M.build_knn_graphs([a.T, b.T], k=6, distance=M.SqEuclidean())
    assert len(graphs) == 2 and graphs[1].neighbors[0] == [2, 3, 4, 5, 6, 7]


def test_full_size_batch_equals_single_graphs_and_replays(gpu_lib):
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib

    clouds = _clouds(64, 2000, 50000, 32, seed=0)
    offs = np.zeros(65, np.int64)
    offs[1:] = np.cumsum([len(c) for c in clouds])
    X = torch.from_numpy(np.concatenate(clouds)).cuda()
    N = int(offs[-1])
    k = 15
    p = _lib.params(_lib.METRIC_SQEUCLIDEAN, k, _lib.PREC_FP32)
    outs = []
    for rep in range(3):  # autotune + capture, then replays
        ids = torch.empty((N, k), dtype=torch.int32, device="cuda")
        d = torch.empty((N, k), dtype=torch.float32, device="cuda")
        r = _lib.KnnReport()
        _lib.check(gpu_lib.mann_knn_graph_batched_device(p, X.data_ptr(), offs.ctypes.data, 64, 32, 0,
                                                         ids.data_ptr(), d.data_ptr(), r, 0))
        torch.cuda.synchronize()
        outs.append((ids.cpu().numpy(), d.cpu().numpy()))
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0]) and np.array_equal(o[1].view(np.uint32), outs[0][1].view(np.uint32))
    ids, d = outs[0]
    bf = M.BruteForceIndex(32, 1, M.SqEuclidean())
    for c in range(0, 64, 9):
        cl = clouds[c]
        bf.n_points = len(cl)
        i1, d1 = M.knn_graph_arrays(bf, cl.T, k)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i1), c
        assert np.array_equal(d[offs[c]:offs[c + 1]].view(np.uint32), d1.view(np.uint32)), c


def test_batched_validation(gpu_lib):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0)
    a = rng.standard_normal((4, 10)).astype(np.float32)
    b = rng.standard_normal((4, 3)).astype(np.float32)
    with pytest.raises(M.ArgumentError):
        M.knn_graph_batched_arrays([a, b], 3)  # k > 3 - 1
    M.knn_graph_batched_arrays([a, b], 3, include_self=True)
    with pytest.raises(M.ArgumentError):
        M.knn_graph_batched_arrays([a, np.zeros((4, 0), np.float32)], 2)
    with pytest.raises(M.ArgumentError):
        M.knn_graph_batched_arrays([a], 2, distance=M.CosineDist())


@pytest.mark.parametrize("metric,d,k", [(1, 32, 15), (0, 7, 5), (1, 12, 23), (1, 40, 10)])
def test_batched_bf16_form_equals_oracle_per_set(gpu_lib, orc, metric, d, k):
    """The tensor-core form of the batched graphs (one segmented pass over
    every set's (block, tile) items, exact FP32 rerank, exact re-scan of
    uncertified rows within their own set) gives each set the oracle's graph."""
    import manifoldann_gb300 as M

    clouds = _clouds(9, 26, 3000, d, seed=100 + d)
    clouds.append(np.random.default_rng(d).standard_normal((28, d)).astype(np.float32))  # below the list depth
    dist = M.SqEuclidean() if metric == 1 else M.Euclidean()
    ids, dists, offs, rep = M.knn_graph_batched_arrays([c.T for c in clouds], k, distance=dist, report=True,
                                                       precision="bf16")
    assert rep["precision_used"] == 1
    for c, cl in enumerate(clouds):
        i_o, d_o = orc.knn_graph_f32(cl, k, metric)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i_o), c
        assert np.array_equal(dists[offs[c]:offs[c + 1]].view(np.uint32), d_o.view(np.uint32)), c


@pytest.mark.parametrize("metric,d,k", [(1, 32, 15), (0, 12, 9)])
def test_batched_fp16_form_equals_oracle_per_set(gpu_lib, orc, metric, d, k):
    import manifoldann_gb300 as M

    clouds = _clouds(7, 26, 3000, d, seed=200 + d)
    dist = M.SqEuclidean() if metric == 1 else M.Euclidean()
    ids, dists, offs, rep = M.knn_graph_batched_arrays([c.T for c in clouds], k, distance=dist, report=True,
                                                       precision="fp16")
    assert rep["precision_used"] == 4
    for c, cl in enumerate(clouds):
        i_o, d_o = orc.knn_graph_f32(cl, k, metric)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i_o), c
        assert np.array_equal(dists[offs[c]:offs[c + 1]].view(np.uint32), d_o.view(np.uint32)), c


def test_batched_bf16_form_ties_duplicates_and_full_size(gpu_lib, orc):
    import manifoldann_gb300 as M

    g = np.stack(np.meshgrid(np.arange(6), np.arange(5), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    a = np.concatenate([g, g[:17]]).astype(np.float32)
    b = (np.arange(40, dtype=np.float32)[:, None] * np.ones((1, 3), np.float32))
    ids, dists, offs = M.knn_graph_batched_arrays([a.T, b.T], 6, distance=M.SqEuclidean(), precision="bf16")
    for c, cl in enumerate((a, b)):
        i_o, d_o = orc.knn_graph_f32(cl, 6, 1)
        assert np.array_equal(ids[offs[c]:offs[c + 1]], i_o)
        assert np.array_equal(dists[offs[c]:offs[c + 1]], d_o)
    clouds = _clouds(64, 2000, 50000, 32, seed=0)
    i32, d32, o32 = M.knn_graph_batched_arrays([c.T for c in clouds], 15, distance=M.SqEuclidean())
    for _ in range(2):  # the second call runs the tuned admission depth
        ib, db, ob, rep = M.knn_graph_batched_arrays([c.T for c in clouds], 15, distance=M.SqEuclidean(),
                                                     precision="bf16", report=True)
        assert np.array_equal(ib, i32) and np.array_equal(db.view(np.uint32), d32.view(np.uint32))
        assert rep["rows_fallback"] <= len(ib) // 100, rep

