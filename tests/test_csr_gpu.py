"""Undirected kNN graph as CSR on the GPU against the reference's set-based
_symmetrize_adjacency (restated on the host in graphs.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_union(ids):
    from manifoldann_gb300.graphs import _symmetrize_adjacency

    adj = [[int(j) + 1 for j in row if j >= 0] for row in ids]
    return _symmetrize_adjacency(adj, len(ids))


def _csr_lists(offs, cols):
    return [(cols[offs[i]:offs[i + 1]].astype(np.int64) + 1).tolist() for i in range(len(offs) - 1)]


def test_union_matches_host_with_gaps_and_self(gpu_lib):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0)
    n, k = 5000, 10
    ids = rng.integers(0, n, size=(n, k)).astype(np.int32)
    ids[rng.random(ids.shape) < 0.05] = -1
    ids[::7, 0] = np.arange(0, n, 7)  # self entries (include_self graphs)
    offs, cols = M.knn_graph_symmetrize_csr(ids)
    assert _csr_lists(offs, cols) == _host_union(ids)


def test_hub_rows_take_the_block_path(gpu_lib):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(1)
    n, k = 6000, 8
    ids = rng.integers(0, n, size=(n, k)).astype(np.int32)
    ids[:, 0] = 0  # every vertex points at 0: row 0 holds n distinct neighbours
    ids[:3000, 1] = 1
    offs, cols = M.knn_graph_symmetrize_csr(ids)
    assert _csr_lists(offs, cols) == _host_union(ids)
    big = np.zeros((20000, 2), np.int32)
    big[:, 1] = np.arange(20000) % 97
    with pytest.raises(M.ArgumentError):
        M.knn_graph_symmetrize_csr(big)


@pytest.mark.parametrize("include_self", [False, True])
def test_undirected_build_knn_graph(gpu_lib, include_self):
    import manifoldann_gb300 as M
    from manifoldann_gb300.graphs import _symmetrize_adjacency

    rng = np.random.default_rng(2)
    data = rng.standard_normal((16, 3000)).astype(np.float32)
    idx = M.build_index(M.BruteForceIndex, data, distance=M.SqEuclidean())
    g_dir = M.build_knn_graph(idx, data, k=8, include_self=include_self)
    g_und = M.build_knn_graph(idx, data, k=8, include_self=include_self, directed=False)
    assert g_und.neighbors == _symmetrize_adjacency(g_dir.neighbors, 3000)
    assert g_und.k == max(len(r) for r in g_und.neighbors)


def test_full_size_union(gpu_lib):
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic

    X = synthetic.quantized_mixture(60000, 784, seed=1)
    idx = M.build_index(M.BruteForceIndex, X.T, distance=M.SqEuclidean())
    ids, _ = M.knn_graph_arrays(idx, X.T, 10, precision="auto")
    offs, cols = M.knn_graph_symmetrize_csr(ids)
    assert _csr_lists(offs, cols) == _host_union(ids)
    assert np.all(np.diff(offs) >= 10)
