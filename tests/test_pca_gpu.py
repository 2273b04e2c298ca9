"""Batched local PCA on the GPU against the FP64 oracle (eigenvalues,
principal subspaces, chosen dimensions), the reference's PCA test cases, and
a full-size run over every node of the 64-cloud kNN graphs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _projector(B):
    return B @ B.T


@pytest.mark.parametrize("d,k,fixed", [(3, 15, 2), (8, 15, None), (32, 15, 2), (100, 20, 3), (16, 32, None),
                                       (40, 5, None)])
def test_local_pca_matches_oracle(gpu_lib, d, k, fixed):
    import manifoldann_gb300 as M
    from oracle import pca

    rng = np.random.default_rng(d * 100 + k)
    n, m = 3000, 400
    scales = np.exp(rng.uniform(-2, 1, size=d))
    X = (rng.standard_normal((n, d)) * scales).astype(np.float32)
    centres = rng.choice(n, m, replace=False)
    nbrs = np.stack([rng.choice(n, k, replace=False) for _ in range(m)])
    method = M.PCAMethod(intrinsic_dim=fixed, min_variance_ratio=0.9)
    dims, eig, basis = M.fit_geometries(method, X.T, nbrs + 1, centers=centres + 1)
    checked = 0
    for i in range(m):
        dim_o, vals_o, B_o = pca.fit_pca(X[centres[i]], X[nbrs[i]], intrinsic_dim=fixed, min_variance_ratio=0.9)
        assert dims[i] == dim_o, (i, dims[i], dim_o)
        lmax = vals_o[0] if vals_o.size else 1.0
        assert np.allclose(eig[i, :dim_o], vals_o, rtol=2e-4, atol=2e-5 * lmax), i
        B = basis[i, :dim_o].T.astype(np.float64)
        assert np.allclose(B.T @ B, np.eye(dim_o), atol=1e-4)
        # compare the subspace where the spectrum has a gap at the cut
        _, full, _ = pca.fit_pca(X[centres[i]], X[nbrs[i]], intrinsic_dim=min(d, k))
        if dim_o < full.size and full[dim_o - 1] - full[dim_o] > 1e-2 * full[0]:
            assert np.abs(_projector(B) - _projector(B_o)).max() < 5e-3, i
            checked += 1
    assert checked > m // 4


def test_local_pca_reference_cases_and_edges(gpu_lib):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(42)
    xy = rng.standard_normal((2, 30))
    data = np.vstack([xy, 0.5 * xy[0] + 0.3 * xy[1]]).astype(np.float32)  # d x n
    g = M.fit_geometry(M.PCAMethod(intrinsic_dim=2), data, 1, range(2, 31))
    normal = np.array([0.5, 0.3, -1.0]) / np.linalg.norm([0.5, 0.3, -1.0])
    assert M.intrinsic_dimension(g) == 2 and g.basis.shape == (3, 2)
    assert np.abs(g.basis.T @ normal).max() < 1e-4
    t = rng.standard_normal(20)
    direction = np.array([1.0, 2.0, 3.0]) / np.linalg.norm([1.0, 2.0, 3.0])
    line = np.outer(direction, t).astype(np.float32)
    g = M.fit_geometry(M.PCAMethod(intrinsic_dim=1), line, 1, range(2, 21))
    assert abs(g.basis[:, 0] @ direction) > 0.99
    # auto dimension (pca_tests.jl:94-108 with 31 neighbours: the GPU fit takes up to 32)
    noisy = np.vstack([rng.standard_normal((2, 32)) * 10, rng.standard_normal((1, 32)) * 0.01]).astype(np.float32)
    assert M.intrinsic_dimension(M.fit_geometry(M.PCAMethod(min_variance_ratio=0.99), noisy, 1, range(2, 33))) == 2
    # a query point as the centre (pca_tests.jl:112-128)
    q = rng.standard_normal(3).astype(np.float32)
    g = M.fit_geometry(M.PCAMethod(intrinsic_dim=2), data, q, range(1, 11))
    assert np.allclose(g.center, q) and g.basis.shape == (3, 2)
    # fewer than two neighbours: identity basis
    dims, eig, basis = M.fit_geometries(M.PCAMethod(intrinsic_dim=2), data, np.array([[5, 0, 0]]), centers=[1])
    assert dims[0] == 2 and np.allclose(basis[0, :2], np.eye(3)[:2]) and np.allclose(eig[0, :2], 1.0)
    # round trip on the tangent space
    g = M.fit_geometry(M.PCAMethod(intrinsic_dim=2), data, 1, range(2, 31))
    y = M.project(g, data[:, 7])
    assert np.allclose(M.reconstruct(g, y), data[:, 7], atol=1e-4)


def test_local_pca_full_graph(gpu_lib):
    import torch

    import manifoldann_gb300 as M
    from manifoldann_gb300 import _lib, synthetic
    from oracle import pca

    clouds = synthetic.manifold_clouds(64, 2000, 50000, 32, seed=0)
    ids, _, offs = M.knn_graph_batched_arrays([c.T for c in clouds], 15, distance=M.SqEuclidean())
    X = np.concatenate(clouds)
    N = len(X)
    glob = ids + np.repeat(offs[:-1], np.diff(offs))[:, None]  # local -> global ids
    Xd = torch.from_numpy(X).cuda()
    nb = torch.from_numpy(glob.astype(np.int32)).cuda()
    cen = torch.arange(N, dtype=torch.int32, device="cuda")
    dims = torch.empty(N, dtype=torch.int32, device="cuda")
    eig = torch.empty((N, 15), dtype=torch.float32, device="cuda")
    basis = torch.empty((N, 15, 32), dtype=torch.float32, device="cuda")
    p = _lib.PcaParams(2, 0, 0.95)
    _lib.check(gpu_lib.mann_local_pca_device(p, Xd.data_ptr(), N, 32, cen.data_ptr(), None, N, nb.data_ptr(), 15, 15,
                                             dims.data_ptr(), eig.data_ptr(), basis.data_ptr(), 0))
    torch.cuda.synchronize()
    dims, eig, basis = dims.cpu().numpy(), eig.cpu().numpy(), basis.cpu().numpy()
    assert np.all(dims == 2)
    B = basis[:, :2, :]
    gram = np.einsum("nid,njd->nij", B, B)
    assert np.abs(gram - np.eye(2)).max() < 1e-4
    rng = np.random.default_rng(1)
    for i in rng.choice(N, 300, replace=False):
        _, vals_o, B_o = pca.fit_pca(X[i], X[glob[i]], intrinsic_dim=2)
        assert np.allclose(eig[i, :2], vals_o, rtol=1e-3, atol=1e-7)


@pytest.mark.parametrize("rule", [0, 1, 2, 3, 4])
def test_edge_weights_match_oracle(gpu_lib, rule):
    import manifoldann_gb300 as M
    from oracle import pca

    from manifoldann_gb300 import synthetic

    clouds = synthetic.manifold_clouds(3, 800, 1500, 16, seed=rule)
    X = np.concatenate(clouds)
    ids, _, offs = M.knn_graph_batched_arrays([c.T for c in clouds], 10, distance=M.SqEuclidean())
    glob = (ids + np.repeat(offs[:-1], np.diff(offs))[:, None]).astype(np.int64)
    glob[5, 3] = -1  # a missing edge gives NaN
    method = M.PCAMethod(intrinsic_dim=2)
    dims, eig, basis = M.fit_geometries(method, X.T, np.where(glob >= 0, glob + 1, 0),
                                        centers=np.arange(len(X)) + 1)
    rules = [M.EuclideanChord(), M.TangentProjectedSourceOnly(), M.TangentProjectedSymmetricMean(),
             M.TangentProjectedSymmetricMax(), M.CurvatureFreeSymmetric()]
    w, neg = M.compute_edge_weights(rules[rule], X.T, np.where(glob >= 0, glob + 1, 0), dims, basis)
    bases = [basis[i].T.astype(np.float64) for i in range(len(X))]
    w_o, neg_o = pca.edge_weights(rule, X, glob, bases, dims)
    assert np.isnan(w[5, 3]) and np.isnan(w_o[5, 3])
    ok = ~np.isnan(w_o)
    assert np.allclose(w[ok], w_o[ok], rtol=1e-4, atol=1e-6)
    assert neg == neg_o
    if rule == 0:
        with pytest.raises(M.ArgumentError):
            M.compute_edge_weights(M.TangentProjectedSourceOnly(), X.T, glob + 1)
