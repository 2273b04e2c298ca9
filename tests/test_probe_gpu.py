"""Learned coarse probe on the GPU: forward scores and gradients of the
hand-written tcgen05 training kernels against the FP64 oracle (with the GPU's
BF16 rounding points), the top-nprobe selection, deterministic training, and
what the trained network gains over centroid routing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(dims, prior, seed=0, C=None, params=None, **kw):
    import manifoldann_gb300 as M

    din, h1, h2, nout = dims
    return M.ProbeModel(din, nout, (h1, h2), use_prior=prior, centroids=C, seed=seed, params=params, **kw)


def _rand_params(dims, rng, scale=1.0, theta=0.0):
    from oracle import probe as P

    L = P.layout(*dims)
    p = np.zeros(L["total"], np.float32)
    din, h1, h2, nout = dims
    for name, fan in (("w1", din), ("b1", din), ("w2", h1), ("b2", h1), ("w3", h2), ("b3", h2)):
        a, b = L[name]
        p[a:b] = rng.uniform(-1, 1, b - a) * scale / np.sqrt(fan)
    p[-1] = theta
    return p


def _blocks(dims):
    from oracle import probe as P

    L = P.layout(*dims)
    return [(k, L[k]) for k in ("w1", "b1", "w2", "b2", "w3", "b3")]


@pytest.mark.parametrize("dims,n", [((40, 96, 160, 200), 300), ((128, 512, 512, 4096), 256)])
def test_scores_match_oracle(gpu_lib, dims, n):
    from oracle import probe as P

    rng = np.random.default_rng(dims[0])
    params = _rand_params(dims, rng, scale=2.0)
    X = rng.standard_normal((n, dims[0])).astype(np.float32)
    m = _model(dims, False, params=params)
    S = m.scores(X)
    S_o = P.scores(params, dims, X)
    err = np.abs(S - S_o).max() / np.abs(S_o).max()
    assert err < 5e-3, err
    assert np.array_equal(m.params(), params)


@pytest.mark.parametrize("dims,n,prior", [((40, 96, 160, 200), 300, False), ((40, 96, 160, 200), 300, True),
                                          ((128, 512, 512, 4096), 256, True)])
def test_gradients_match_oracle(gpu_lib, dims, n, prior):
    from oracle import probe as P

    rng = np.random.default_rng(7 + prior)
    params = _rand_params(dims, rng, scale=2.0, theta=np.log(0.05))
    X = rng.standard_normal((n, dims[0])).astype(np.float32)
    C = rng.standard_normal((dims[3], dims[0])).astype(np.float32) if prior else None
    labels = rng.integers(-1, dims[3], size=(n, 10)).astype(np.int32)
    labels[3, :] = -1  # a row without labels contributes nothing
    m = _model(dims, prior, C=C, params=params)
    loss, g = m.grad(X, labels)
    loss_o, g_o = P.forward_backward(params, dims, X, labels, C)
    assert abs(loss - loss_o) <= 1e-4 * abs(loss_o) + 1e-5
    for name, (a, b) in _blocks(dims):
        rel = np.linalg.norm(g[a:b] - g_o[a:b]) / max(np.linalg.norm(g_o[a:b]), 1e-30)
        assert rel < 2e-2, (name, rel)
    if prior:
        assert abs(g[-1] - g_o[-1]) <= 2e-3 * abs(g_o[-1]) + 1e-6
    else:
        assert g[-1] == 0.0


def test_route_topk_order_and_ties(gpu_lib):
    import torch

    dims = (64, 128, 128, 1000)
    rng = np.random.default_rng(3)
    params = _rand_params(dims, rng, scale=3.0)
    X = rng.standard_normal((777, 64)).astype(np.float32)
    m = _model(dims, False, params=params)
    S = m.scores(X)
    qd = torch.from_numpy(X).cuda()
    order = np.stack([np.lexsort((np.arange(1000), -S[i])) for i in range(777)])
    e = np.exp(S - S.max(1, keepdims=True))
    for nprobe in (1, 3, 8, 13, 16, 37, 128):  # warp kernels up to 16, radix select above
        pr = torch.empty((777, nprobe), dtype=torch.int32, device="cuda")
        cov = torch.empty(777, dtype=torch.float32, device="cuda")
        m.route_device(qd, nprobe, pr, cov)
        torch.cuda.synchronize()
        want = order[:, :nprobe]
        assert np.array_equal(pr.cpu().numpy(), want), nprobe
        cov_o = np.take_along_axis(e, want, 1).sum(1) / e.sum(1)
        assert np.allclose(cov.cpu().numpy(), cov_o, rtol=1e-4, atol=1e-6), nprobe
    # all-equal scores: ties go to the lower list id
    z = np.zeros_like(params)
    mz = _model(dims, False, params=z)
    mz.route_device(qd[:5], 9, pr_t := torch.empty((5, 9), dtype=torch.int32, device="cuda"))
    torch.cuda.synchronize()
    assert (pr_t.cpu().numpy() == np.arange(9)).all()


@pytest.mark.parametrize("nout", [64, 100, 576, 4100])
def test_route_topk_uneven_list_counts(gpu_lib, nout):
    """List counts whose float4 groups do not fill whole 128-group passes
    (nout mod 512 in 1..124): every lane still takes the warp-wide exchange
    the same number of times, so the order equals the oracle's."""
    import torch

    dims = (32, 128, 128, nout)
    rng = np.random.default_rng(nout)
    params = _rand_params(dims, rng, scale=3.0)
    X = rng.standard_normal((301, 32)).astype(np.float32)
    m = _model(dims, False, params=params)
    S = m.scores(X)
    qd = torch.from_numpy(X).cuda()
    order = np.stack([np.lexsort((np.arange(nout), -S[i])) for i in range(len(X))])
    e = np.exp(S - S.max(1, keepdims=True))
    for nprobe in (1, 4, 16):
        pr = torch.empty((len(X), nprobe), dtype=torch.int32, device="cuda")
        cov = torch.empty(len(X), dtype=torch.float32, device="cuda")
        m.route_device(qd, nprobe, pr, cov)
        torch.cuda.synchronize()
        want = order[:, :nprobe]
        assert np.array_equal(pr.cpu().numpy(), want), nprobe
        cov_o = np.take_along_axis(e, want, 1).sum(1) / e.sum(1)
        assert np.allclose(cov.cpu().numpy(), cov_o, rtol=1e-4, atol=1e-6), nprobe


def test_training_is_deterministic_and_lowers_loss(gpu_lib):
    dims = (32, 128, 128, 64)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((3000, 32)).astype(np.float32)
    C = rng.standard_normal((64, 32)).astype(np.float32)
    d2 = ((X[:, None, :] - C[None]) ** 2).sum(-1)
    labels = np.argsort(d2, 1)[:, :3].astype(np.int32)
    out = []
    for _ in range(2):
        m = _model(dims, True, C=C, seed=11, batch=512, lr=3e-3)
        loss = m.train(X, labels, 4)
        out.append((loss, m.params()))
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][0][-1] < out[0][0][0]


def test_learned_routing_against_centroid_routing(gpu_lib, orc):
    """Recall@10 at equal nprobe: the trained probe (with the distance prior)
    stays at least level with centroid routing (TopKRouting on the KMeans
    distances), and training lifts the plain MLP far above its untrained
    self; the scan of the learned probes is exact."""
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic

    X = synthetic.anisotropic_clusters(40000, 32, seed=21, clusters=64)
    TQ = synthetic.anisotropic_clusters(20000, 32, seed=22, clusters=64)
    Q = synthetic.anisotropic_clusters(1000, 32, seed=23, clusters=64)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=256, seed=4)
    r = M.LearnedProbeRouting.train(idx, X.T, TQ.T, k=4, hidden=(256, 256), epochs=12, batch=1024,
                                    lr=2e-3, seed=3)
    assert r.loss_curve[-1] < r.loss_curve[0]
    truth, _ = orc.knn_f32(X, Q, 10, 0)

    def recall(ids):
        return np.mean([len(set(ids[i]) & set(truth[i])) / 10 for i in range(len(Q))])

    rec_l, rec_c = [], []
    for npb in (1, 2, 4):
        ids_l, d_l = M.ivf_search_learned(idx, r, X.T, Q.T, 10, nprobe=npb)
        ids_c, _ = idx.search_arrays(X.T, Q.T, 10, nprobe=npb)
        rec_l.append(recall(ids_l))
        rec_c.append(recall(ids_c))
        probes = r.select(Q.T, npb)
        ids_o, d_o = orc.ivf_scan_f32(X, idx.list_offsets, idx.list_ids, Q, probes, 10, 0)
        assert np.array_equal(ids_l, ids_o)
        assert np.array_equal(d_l.view(np.uint32), d_o.view(np.uint32))
    assert sum(rec_l) >= sum(rec_c) - 0.006, (rec_l, rec_c)
    untrained = M.LearnedProbeRouting(2, M.ProbeModel(32, 256, (256, 256), use_prior=False, seed=3))
    plain = M.LearnedProbeRouting.train(idx, X.T, TQ.T, k=2, hidden=(256, 256), epochs=12, batch=1024,
                                        lr=2e-3, use_prior=False, seed=3)
    r_u = recall(M.ivf_search_learned(idx, untrained, X.T, Q.T, 10)[0])
    r_p = recall(M.ivf_search_learned(idx, plain, X.T, Q.T, 10)[0])
    assert r_p > r_u + 0.3, (r_p, r_u)
