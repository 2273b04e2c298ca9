"""IVF-Flat on the GPU against the oracle: the inverted lists (a partition of
the points by exact nearest centroid, ascending ids per list), the routing
(exact top-nprobe centroids), and the list scan (ids and distance bits equal
to the oracle's scan of the same probes)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, d, seed, clusters=40):
    from manifoldann_gb300 import synthetic

    return synthetic.anisotropic_clusters(n, d, seed=seed, clusters=clusters)  # [n][d]


@pytest.mark.parametrize("metric", [0, 1])
def test_build_lists_partition_by_nearest_centroid(gpu_lib, orc, metric):
    import manifoldann_gb300 as M

    X = _data(20000, 32, 1)
    cm = M.Euclidean() if metric == 0 else M.SqEuclidean()
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=64, nprobe=8, centroid_metric=cm, seed=3)
    assert idx.nlist == 64 and idx.default_nprobe == 8 and idx.dimension == 32
    offs, ids = idx.list_offsets, idx.list_ids
    assert offs[0] == 0 and offs[-1] == len(X) and np.all(np.diff(offs) >= 0)
    assert np.array_equal(np.sort(ids), np.arange(len(X)))
    for c in range(64):
        seg = ids[offs[c]:offs[c + 1]]
        assert np.all(np.diff(seg) > 0)
    a_o, _ = orc.kmeans_assign_f64(X, idx.centroids.T, metric)
    owner = np.empty(len(X), np.int64)
    for c in range(64):
        owner[ids[offs[c]:offs[c + 1]]] = c
    assert np.array_equal(owner, a_o)
    assert np.allclose(idx.centroid_norms, (idx.centroids.T.astype(np.float64) ** 2).sum(1), rtol=1e-5)
    lists = idx.lists
    assert sum(len(l) for l in lists) == len(X) and min(min(l) for l in lists if l) == 1


@pytest.mark.parametrize("metric,centroid_metric,d,k,nprobe",
                         [(0, 0, 32, 10, 8), (1, 0, 128, 10, 16), (0, 1, 96, 32, 5), (1, 1, 17, 64, 3)])
def test_search_equals_oracle_scan_of_exact_routing(gpu_lib, orc, metric, centroid_metric, d, k, nprobe):
    import manifoldann_gb300 as M

    X = _data(30000, d, 2 + d)
    Q = _data(700, d, 900 + d)
    dist = M.Euclidean() if metric == 0 else M.SqEuclidean()
    cm = M.Euclidean() if centroid_metric == 0 else M.SqEuclidean()
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=100, nprobe=nprobe, distance=dist,
                        centroid_metric=cm, seed=5)
    ids, dists = idx.search_arrays(X.T, Q.T, k)
    probes, _ = orc.knn_f32(idx.centroids.T, Q, nprobe, centroid_metric)
    ids_o, d_o = orc.ivf_scan_f32(X, idx.list_offsets, idx.list_ids, Q, probes, k, metric)
    assert np.array_equal(ids, ids_o)
    assert np.array_equal(dists.view(np.uint32), d_o.view(np.uint32))


def test_scan_given_probes_with_unused_slots(gpu_lib, orc):
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib

    X = _data(12000, 48, 7)
    Q = _data(300, 48, 8)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=50, seed=1)
    rng = np.random.default_rng(0)
    nprobe, k = 6, 12
    probes = np.stack([rng.choice(50, nprobe, replace=False) for _ in range(len(Q))]).astype(np.int32)
    probes[rng.random(probes.shape) < 0.3] = -1
    probes[5, :] = -1  # a query with no list at all
    dev = torch.device("cuda:0")
    Xd = torch.from_numpy(X).to(dev)
    Qd = torch.from_numpy(Q).to(dev)
    Pd = torch.from_numpy(probes).to(dev)
    od = torch.from_numpy(idx.list_offsets).to(dev)
    idd = torch.from_numpy(idx.list_ids).to(dev)
    oi = torch.empty((len(Q), k), dtype=torch.int32, device=dev)
    odist = torch.empty((len(Q), k), dtype=torch.float32, device=dev)
    p = _lib.params(0, k, _lib.PREC_FP32, 0, 0)
    _lib.check(gpu_lib.mann_ivf_scan_device(p, Pd.data_ptr(), nprobe, Xd.data_ptr(), len(X), 48, 50,
                                            od.data_ptr(), idd.data_ptr(), Qd.data_ptr(), len(Q),
                                            oi.data_ptr(), odist.data_ptr(), 0))
    torch.cuda.synchronize()
    ids_o, d_o = orc.ivf_scan_f32(X, idx.list_offsets, idx.list_ids, Q, probes, k, 0)
    assert np.array_equal(oi.cpu().numpy(), ids_o)
    assert np.array_equal(odist.cpu().numpy().view(np.uint32), d_o.view(np.uint32))
    assert np.all(oi.cpu().numpy()[5] == -1)


def test_short_lists_pad_and_query_truncates(gpu_lib, orc):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(4)
    X = rng.standard_normal((40, 8)).astype(np.float32)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=8, nprobe=1, seed=2)
    q = rng.standard_normal(8).astype(np.float32)
    k = 30
    ids, dists = idx.search_arrays(X.T, q, k)
    probes, _ = orc.knn_f32(idx.centroids.T, q[None], 1, 0)
    ids_o, d_o = orc.ivf_scan_f32(X, idx.list_offsets, idx.list_ids, q[None], probes, k, 0)
    assert np.array_equal(ids, ids_o)
    avail = idx.list_offsets[probes[0, 0] + 1] - idx.list_offsets[probes[0, 0]]
    assert avail < k and np.all(ids[0, avail:] == -1) and np.all(np.isinf(dists[0, avail:]))
    got = M.query(idx, X.T, q, k)
    assert len(got) == avail and [n.id for n in got] == (ids[0, :avail] + 1).tolist()


def test_nprobe_all_lists_is_exact_and_recall_grows(gpu_lib, orc):
    import manifoldann_gb300 as M

    X = _data(20000, 64, 11, clusters=60)
    Q = _data(400, 64, 12, clusters=60)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=64, seed=9)
    truth, td = orc.knn_f32(X, Q, 10, 0)
    ids, dists = idx.search_arrays(X.T, Q.T, 10, nprobe=64)
    assert np.array_equal(ids, truth)
    assert np.array_equal(dists.view(np.uint32), td.view(np.uint32))
    ids_big, _ = idx.search_arrays(X.T, Q.T, 10, nprobe=1000)  # clamped to nlist
    assert np.array_equal(ids_big, truth)
    rec = []
    for npb in (1, 4, 16):
        got, _ = idx.search_arrays(X.T, Q.T, 10, nprobe=npb)
        rec.append(np.mean([len(set(got[i]) & set(truth[i])) / 10 for i in range(len(Q))]))
    assert rec[0] <= rec[1] <= rec[2] and rec[2] > 0.9


def test_batch_query_matches_single_queries(gpu_lib):
    # test/unit/indices/abstract_batch_query_tests.jl:9-61 (IVFFlat case)
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0xBA7CE5)
    data = rng.standard_normal((16, 1000)).astype(np.float32)
    queries = rng.standard_normal((16, 80)).astype(np.float32)
    idx = M.build_index(M.IVFFlatIndex, data, nlist=8, nprobe=4)
    ref = [M.query(idx, data, queries[:, i], 5) for i in range(80)]
    got = M.query(idx, data, queries, 5)
    assert len(got) == 80
    for i in range(80):
        assert [n.id for n in got[i]] == [n.id for n in ref[i]]
    got_vv = M.query(idx, data, [queries[:, i].copy() for i in range(80)], 5)
    for i in range(80):
        assert [n.id for n in got_vv[i]] == [n.id for n in ref[i]]


def test_ivf_validation(gpu_lib):
    import manifoldann_gb300 as M

    X = np.zeros((4, 10), np.float32)
    with pytest.raises(M.ArgumentError):
        M.build_index(M.IVFFlatIndex, X, nlist=0)
    with pytest.raises(M.ArgumentError):
        M.build_index(M.IVFFlatIndex, np.zeros((4, 0), np.float32), nlist=2)
    idx = M.build_index(M.IVFFlatIndex, np.random.default_rng(0).standard_normal((4, 10)).astype(np.float32),
                        nlist=2)
    with pytest.raises(M.DimensionMismatch):
        idx.query(np.zeros((5, 10), np.float32), np.zeros(5, np.float32), 3)
    with pytest.raises(M.DimensionMismatch):
        idx.query(np.zeros((4, 10), np.float32), np.zeros(3, np.float32), 3)


def test_index_and_probe_persist(gpu_lib, tmp_path):
    import manifoldann_gb300 as M

    X = _data(8000, 24, 31)
    Q = _data(200, 24, 32)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=32, nprobe=3, distance=M.SqEuclidean(), seed=2)
    idx.save(tmp_path / "ivf.npz")
    idx2 = M.IVFFlatIndex.load(tmp_path / "ivf.npz")
    a, da = idx.search_arrays(X.T, Q.T, 7)
    b, db = idx2.search_arrays(X.T, Q.T, 7)
    assert np.array_equal(a, b) and np.array_equal(da, db)
    assert idx2.distance == idx.distance and idx2.default_nprobe == 3
    r = M.LearnedProbeRouting.train(idx, X.T, _data(3000, 24, 33).T, k=3, hidden=(128, 128), epochs=2, seed=1)
    r.model.save(tmp_path / "probe.npz")
    m2 = M.ProbeModel.load(tmp_path / "probe.npz")
    assert np.array_equal(m2.params(), r.model.params())
    r2 = M.LearnedProbeRouting(3, m2)
    assert np.array_equal(M.ivf_search_learned(idx, r, X.T, Q.T, 7)[0], M.ivf_search_learned(idx2, r2, X.T, Q.T, 7)[0])
