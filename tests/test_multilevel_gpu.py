"""MultiLevelIndex with a KMeans transform and BruteForce children (the
reference's src/indices/multilevel/), and the candidate lists of
build_weighted_graph (src/graphs/weighted_knn_graph.jl:497-567).

* batch == per-query single queries (port of
  test/unit/indices/abstract_batch_query_tests.jl:133-156, with BruteForce
  children in place of HNSW, which is outside this library), for the matrix
  and the vector-of-vectors inputs;
* SimpleMerge and DisjointMerge against the oracle: the probed children from
  the FP32 centroid distances (partialsortperm order), each child's exact
  FP32 top-k (BruteForceIndex on the child's points), merged by the
  reference's rules (merge.jl:79-124 stable sort + dedup; :150-169 bounded
  heap) -- ids and distance bits identical, both GPU engines;
* the candidate lists: query(index, data, x_i, candidate_k + 1), self dropped,
  first candidate_k kept, for every node at once -- equal to the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ml(X, nlist, nprobe, merge, max_iters=25, seed=3):
    import manifoldann_gb300 as M
    from manifoldann_gb300 import multilevel as ML

    cfg = ML.TransformedConfig(M.KMeansTransform(k=nlist, distance=M.Euclidean(), max_iters=max_iters),
                               M.TopKRouting(nprobe), ML.TerminalConfig(M.BruteForceIndex, {"distance": M.SqEuclidean()}))
    return ML.build_multilevel_index(X.T, cfg, merge_strategy=merge, distance=M.SqEuclidean(), seed=seed)


def test_multilevel_batch_matches_single(gpu_lib):
    from manifoldann_gb300 import multilevel as ML

    rng = np.random.default_rng(0xBA7CE5)
    data = rng.standard_normal((16, 1000)).astype(np.float32)
    queries = rng.standard_normal((16, 80)).astype(np.float32)
    k = 5
    ml = _ml(data.T, 4, 2, ML.SimpleMerge(), max_iters=2)
    ref = [ML.multilevel_query(ml, data, queries[:, i], k) for i in range(80)]
    got = ML.multilevel_query(ml, data, queries, k)
    assert len(got) == 80
    for i in range(80):
        assert [n.id for n in got[i]] == [n.id for n in ref[i]]
    got_vv = ML.multilevel_query(ml, data, [queries[:, i].copy() for i in range(80)], k)
    for i in range(80):
        assert [n.id for n in got_vv[i]] == [n.id for n in ref[i]]
    # dimension check even on an empty batch, empty result for k <= 0
    with pytest.raises(Exception):
        ML.multilevel_query(ml, data, np.zeros((15, 0), np.float32), k)
    assert ML.multilevel_query(ml, data, queries[:, :3], 0) == [[], [], []]


def _expected(orc, X, ml, Q, probes, k, merge):
    from manifoldann_gb300 import multilevel as ML
    from manifoldann_gb300.indices import Neighbor

    out = []
    node = ml.root
    for qi in range(len(Q)):
        lists = []
        for c in probes[qi]:
            ids = node.id_mappings[c] - 1
            kk = min(k, len(ids))
            li, ld = orc.knn_f32(X[ids], Q[qi:qi + 1], kk, orc.SQEUCLIDEAN)
            lists.append([Neighbor(int(ids[i]) + 1, float(d)) for i, d in zip(li[0], ld[0]) if i >= 0])
        out.append(ML.merge_results(merge, lists, k))
    return out


@pytest.mark.parametrize("merge_name", ["SimpleMerge", "DisjointMerge"])
def test_multilevel_vs_oracle(gpu_lib, orc, merge_name):
    from manifoldann_gb300 import multilevel as ML
    from manifoldann_gb300 import synthetic

    X = synthetic.anisotropic_clusters(20000, 32, seed=5, clusters=64)
    Q = synthetic.anisotropic_clusters(200, 32, seed=6, clusters=64)
    merge = getattr(ML, merge_name)()
    ml = _ml(X, 64, 4, merge)
    k = 10
    probes = ML._route(ml.root, Q)
    # the routing is the FP32 centroid distances' partialsortperm order
    C = np.ascontiguousarray(ml.root.transform.centroids.T)
    pr_o, _ = orc.knn_f32(C, Q, 4, orc.EUCLIDEAN)
    lookup = ml.root.bucket_lookup
    assert all(np.array_equal(probes[i], lookup[pr_o[i]] - 1) for i in range(len(Q)))
    want = _expected(orc, X, ml, Q, probes, k, merge)
    for engine in ("per_child", "scan"):
        got = ML.multilevel_query(ml, X.T, Q.T, k, engine=engine)
        for i in range(len(Q)):
            assert [n.id for n in got[i]] == [n.id for n in want[i]], (engine, i)
            assert np.array_equal(np.float32([n.dist for n in got[i]]).view(np.uint32),
                                  np.float32([n.dist for n in want[i]]).view(np.uint32)), (engine, i)


def test_weighted_graph_candidate_lists(gpu_lib, orc):
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic
    from oracle import pca as opca

    cl = synthetic.manifold_clouds(1, 3000, 3000, 16, seed=4)[0]
    data = cl.T
    index = M.build_index(M.BruteForceIndex, data, distance=M.SqEuclidean())
    ck = 20
    cand = M.candidate_neighbors(index, data, ck)  # 1-based, [n][ck]
    ids, _ = orc.knn_f32(cl, cl, ck + 1, orc.SQEUCLIDEAN)
    want = np.stack([[j for j in row if j != i][:ck] for i, row in enumerate(ids)]) + 1
    assert np.array_equal(cand, want)
    # build_weighted_graph with candidate_k > k fits every geometry on the candidates
    wg = M.build_weighted_graph(M.PCAMethod(intrinsic_dim=2), index, data, k=8, candidate_k=ck,
                                edge_weight=M.TangentProjectedSourceOnly())
    assert wg.graph_ids.shape == (len(cl), 8)
    for i in (0, 1234, len(cl) - 1):
        _, vals_o, _ = opca.fit_pca(cl[i], cl[cand[i] - 1], intrinsic_dim=2)
        assert np.allclose(wg.eigenvalues[i, :2], vals_o, rtol=1e-3)
    w2, _ = M.compute_edge_weights(M.TangentProjectedSourceOnly(), data, wg.graph_ids + 1, wg.dims, wg.bases)
    assert np.array_equal(np.nan_to_num(w2), np.nan_to_num(wg.edge_weights))
