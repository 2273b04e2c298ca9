"""Device dataset handle (mann_dataset_*): searches over an uploaded point
set equal the host-pointer calls bit for bit, and a re-upload after insert!
(src/indices/bruteforce.jl:82-95) is what later searches see."""
import numpy as np
import pytest

from test_knn_gpu import M_COS, M_EUC, M_SQ, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", [M_SQ, M_EUC, M_COS])
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_dataset_search_equals_host_call(gpu_lib, metric, precision):
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(9000, 96, seed=21)
    q = synthetic.quantized_mixture(300, 96, seed=22)
    dist = {M_EUC: M.Euclidean(), M_SQ: M.SqEuclidean(), M_COS: M.CosineDist()}[metric]
    index = M.build_index(M.BruteForceIndex, base.T, distance=dist)
    ds = M.DeviceDataset(base.T)
    assert ds.shape == (96, 9000)
    a_ids, a_d = M.knn_arrays(index, base.T, q.T, 10, precision=precision)
    b_ids, b_d = M.knn_arrays(index, ds, q.T, 10, precision=precision)
    assert np.array_equal(a_ids, b_ids) and same_bits(a_d, b_d)
    g_ids, g_d = M.knn_graph_arrays(index, base.T, 9, precision=precision)
    h_ids, h_d = M.knn_graph_arrays(index, ds, 9, precision=precision)
    assert np.array_equal(g_ids, h_ids) and same_bits(g_d, h_d)
    ds.close()


def test_dataset_upload_after_insert(gpu_lib, orc):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(5)
    data = rng.standard_normal((24, 500)).astype(np.float32)
    index = M.build_index(M.BruteForceIndex, data, distance=M.SqEuclidean())
    ds = M.DeviceDataset(data)
    q = rng.standard_normal((24, 7)).astype(np.float32)
    more = q[:, :3] + 1e-3  # new points right next to three of the queries
    M.insert(index, more)
    data2 = np.concatenate([data, more], axis=1)
    ds.upload(data2)
    assert ds.shape == (24, 503)
    ids, d = M.knn_arrays(index, ds, q, 4)
    ids_o, d_o = orc.knn_f32(data2.T, q.T, 4, M_SQ)
    assert np.array_equal(ids, ids_o) and same_bits(d, d_o)
    assert [int(i) for i in ids[:3, 0]] == [500, 501, 502]
    with pytest.raises(M.DimensionMismatch):
        ds.upload(np.zeros((5, 10), np.float32))
    ds.close()
    ds.close()  # idempotent


def test_prepared_points_follow_uploads_metrics_and_forms(gpu_lib, orc):
    """A handle keeps its points' prepared tensor-core operand between calls:
    repeated calls, other metrics and forms, graphs, a second handle in
    between and a re-upload of the same size must all give the oracle's
    answer (a stale operand would not)."""
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic

    a = synthetic.anisotropic_clusters(8000, 128, seed=41, clusters=32)
    b = synthetic.anisotropic_clusters(8000, 128, seed=42, clusters=32)  # same shape, other points
    q = synthetic.anisotropic_clusters(250, 128, seed=43, clusters=32)
    dists = {M_SQ: M.SqEuclidean(), M_EUC: M.Euclidean(), M_COS: M.CosineDist()}
    ds = M.DeviceDataset(a.T)
    other = M.DeviceDataset(b.T)
    cur = a
    steps = [(M_SQ, "bf16"), (M_SQ, "bf16"), (M_SQ, "fp16"), (M_COS, "fp16"), (M_SQ, "bf16"), ("other", None),
             (M_SQ, "bf16"), ("upload", None), (M_SQ, "bf16"), (M_COS, "bf16"), ("graph", "fp16"), (M_EUC, "fp16")]
    for metric, prec in steps:
        if metric == "other":
            idx = M.build_index(M.BruteForceIndex, b.T, distance=M.SqEuclidean())
            ids, d = M.knn_arrays(idx, other, q.T, 10, precision="bf16")
            ids_o, d_o = orc.knn_f32(b, q, 10, M_SQ)
        elif metric == "upload":
            ds.upload(b.T)
            cur = b
            continue
        elif metric == "graph":
            idx = M.build_index(M.BruteForceIndex, cur.T, distance=M.SqEuclidean())
            ids, d = M.knn_graph_arrays(idx, ds, 8, precision=prec)
            ids_o, d_o = orc.knn_graph_f32(cur, 8, M_SQ)
        else:
            idx = M.build_index(M.BruteForceIndex, cur.T, distance=dists[metric])
            ids, d = M.knn_arrays(idx, ds, q.T, 10, precision=prec)
            ids_o, d_o = orc.knn_f32(cur, q, 10, metric)
        assert np.array_equal(ids, ids_o), (metric, prec)
        assert same_bits(d, d_o), (metric, prec)
    ds.close()
    other.close()


def test_dataset_argument_errors(gpu_lib):
    import ctypes as C

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib

    lib = _lib.load()
    h = C.c_void_p()
    x = np.zeros((4, 3), np.float32)
    assert lib.mann_dataset_create(x.ctypes.data, 0, 3, C.byref(h)) == 2
    assert lib.mann_dataset_create(None, 4, 3, C.byref(h)) == 2
    ds = M.DeviceDataset(x.T)
    index = M.build_index(M.BruteForceIndex, x.T)
    with pytest.raises(M.ArgumentError):
        M.knn_graph_arrays(index, ds, 4)
    ids, d = M.knn_arrays(index, ds, np.zeros((3, 0), np.float32), 2)
    assert ids.shape == (0, 2) or ids.shape == (0, 0)
    assert lib.mann_dataset_destroy(None) == 0
