"""Parity of the BF16 tensor-core form (MANN_PREC_BF16): certified candidates
reranked in exact FP32 must give exactly the FP32 oracle's answer (ids and
distance bits); with MANN_FLAG_FP64_TIES the ids must equal the FP64 oracle's.
The report's fallback counter must stay near zero -- a wrong tensor-core tile
would otherwise hide behind the exact FP32 fallback."""
import numpy as np
import pytest

from conftest import load_golden
from test_knn_gpu import M_COS, M_EUC, M_SQ, gpu_graph, gpu_knn, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", [M_SQ, M_EUC])
def test_bf16_golden_mixture(gpu_lib, metric, orc):
    g = load_golden("knn_mix_sq_d784")
    base, q = g["base"], g["queries"]
    ids, d, rep = gpu_knn(base, q, 10, metric, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 10, metric)
    assert np.array_equal(ids, ids_o)
    assert same_bits(d, d_o)
    assert rep["precision_used"] == 1
    assert rep["rows_fallback"] <= 2, rep


def test_bf16_fp64_ties_golden(gpu_lib):
    g = load_golden("knn_mix_sq_d784")
    ids, d, rep = gpu_knn(g["base"], g["queries"], 10, M_SQ, precision="bf16", fp64_ties=True,
                          report=True)
    assert np.array_equal(ids, g["ids_f64"])
    # distances are the FP32 ones
    assert np.all(np.abs(d - g["dists_f64"]) <= 1e-5 * np.abs(g["dists_f64"]) + 1e-6)


def test_bf16_graph_golden(gpu_lib):
    g = load_golden("graph_mix_sq_d784")
    ids, d, rep = gpu_graph(g["data"], 10, M_SQ, precision="bf16", report=True)
    assert np.array_equal(ids, g["ids_f32"])
    assert same_bits(d, g["dists_f32"])
    ids64, _ = gpu_graph(g["data"], 10, M_SQ, precision="bf16", fp64_ties=True)
    assert np.array_equal(ids64, g["ids_f64"])


@pytest.mark.parametrize("n,nq,d,k", [(20000, 700, 128, 10), (9000, 300, 256, 20), (5000, 129, 784, 24),
                                      (3000, 40, 200, 1), (777, 33, 96, 16), (300, 5, 130, 24)])
def test_bf16_iid_shapes(gpu_lib, orc, n, nq, d, k):
    rng = np.random.default_rng(n + d)
    base = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((nq, d)).astype(np.float32)
    ids, dist, rep = gpu_knn(base, q, k, M_SQ, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, k, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dist, d_o)
    # i.i.d. Gaussian points are the hard case for BF16 rounding: some rows fall
    # back to the exact scan (the answer is exact either way); a broken tile
    # would make every row fall back
    if d <= 256:
        assert rep["rows_fallback"] <= max(2, nq // 2), rep


def test_bf16_quantized_workload_slice(gpu_lib, orc):
    # the 784-d quantised mixture at 1/6 of its point count, all queries of one batch
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(10000, 784, seed=1)
    q = synthetic.quantized_mixture(500, 784, seed=2)
    ids, d, rep = gpu_knn(base, q, 10, M_SQ, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o) and same_bits(d, d_o)
    assert rep["rows_fallback"] <= 5, rep
    ids64, _ = gpu_knn(base, q, 10, M_SQ, precision="bf16", fp64_ties=True)
    ids_o64, _ = orc.knn_f64(base, q, 10, orc.SQEUCLIDEAN)
    assert np.array_equal(ids64, ids_o64)


def test_bf16_rejects_large_k(gpu_lib):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(0)
    base = rng.standard_normal((500, 128)).astype(np.float32)
    with pytest.raises(M.ArgumentError):
        gpu_knn(base, base[:3], 25, M_SQ, precision="bf16")
    # automatic choice falls back to the FP32 form for large k
    ids, _ = gpu_knn(base, base[:3], 40, M_SQ, precision="auto")
    assert ids.shape == (3, 40)


def test_fp32_form_fp64_ties(gpu_lib, orc):
    g = load_golden("knn_mix_sq_d784")
    ids, _ = gpu_knn(g["base"], g["queries"], 10, M_SQ, precision="fp32", fp64_ties=True)
    assert np.array_equal(ids, g["ids_f64"])
    g = load_golden("knn_iid_cos_d37")
    ids, _ = gpu_knn(g["base"], g["queries"], 20, 2, precision="fp32", fp64_ties=True)
    assert np.array_equal(ids, g["ids_f64"])


def test_bf16_duplicates_certify_or_fall_back(gpu_lib, orc):
    # many identical points: the candidate list cannot be certified, the exact
    # scan answers instead -- still identical to the oracle
    rng = np.random.default_rng(2)
    base = np.repeat(rng.standard_normal((40, 128)).astype(np.float32), 100, axis=0)
    q = base[::97].copy()
    ids, d, rep = gpu_knn(base, q, 10, M_SQ, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    assert np.array_equal(ids, ids_o) and same_bits(d, d_o)


def test_bf16_full_size_equals_fp32_kernel(gpu_lib):
    # N=60,000 quantised 784-d points, 10,000 held-out queries and the self graph:
    # the two GPU forms must agree bit for bit (size-independent property)
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(60000, 784, seed=1)
    q = synthetic.quantized_mixture(10000, 784, seed=2)
    i32, d32 = gpu_knn(base, q, 10, M_SQ, precision="fp32")
    ib, db, rep = gpu_knn(base, q, 10, M_SQ, precision="bf16", report=True)
    assert np.array_equal(i32, ib) and same_bits(d32, db)
    assert rep["rows_fallback"] <= 20, rep
    assert np.all(np.diff(db, axis=1) >= 0)
    g32, gd32 = gpu_graph(base, 10, M_SQ, precision="fp32")
    gb, gdb, rep = gpu_graph(base, 10, M_SQ, precision="bf16", report=True)
    assert np.array_equal(g32, gb) and same_bits(gd32, gdb)
    assert not np.any(gb == np.arange(60000)[:, None])
    assert rep["rows_fallback"] <= 120, rep


@pytest.mark.parametrize("margin", [0, 4, 6, 20])
def test_bf16_admission_depth(gpu_lib, orc, margin):
    # margin 0 = autotuned depth: the first call on a shape runs the full list,
    # later calls the tuned depth (two epilogue warp sets when it is <= 16);
    # explicit margins pick the depth directly
    from manifoldann_gb300 import synthetic

    base = synthetic.quantized_mixture(6000, 784, seed=5)
    q = synthetic.quantized_mixture(300, 784, seed=6)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    g_o, gd_o = orc.knn_graph_f32(base[:3000], 10, orc.SQEUCLIDEAN)
    for _ in range(3):
        ids, d, rep = gpu_knn(base, q, 10, M_SQ, precision="bf16", margin=margin, report=True)
        assert np.array_equal(ids, ids_o) and same_bits(d, d_o)
        gi, gd = gpu_graph(base[:3000], 10, M_SQ, precision="bf16", margin=margin)
        assert np.array_equal(gi, g_o) and same_bits(gd, gd_o)


def test_bf16_seeded_pass(gpu_lib, orc):
    # n >= 32768 points switches on the sampled seed pass; the answer must not change
    from manifoldann_gb300 import synthetic

    base = synthetic.anisotropic_clusters(40000, 128, seed=3, clusters=256)
    q = synthetic.anisotropic_clusters(300, 128, seed=4, clusters=256)
    ids_o, d_o = orc.knn_f32(base, q, 10, orc.SQEUCLIDEAN)
    for _ in range(3):
        ids, d, rep = gpu_knn(base, q, 10, M_SQ, precision="bf16", report=True)
        assert np.array_equal(ids, ids_o) and same_bits(d, d_o)


# ---- cosine: the tensor-core pass on unit-normalised rows, FP32-form cosine rerank

def _angular(n, d, seed):
    from manifoldann_gb300 import synthetic

    return synthetic.angular_clusters(n, d, seed=seed)


@pytest.mark.parametrize("n,nq,d,k", [(20000, 600, 256, 20), (6000, 300, 128, 10), (9000, 200, 200, 24)])
def test_bf16_cosine_equals_oracle(gpu_lib, orc, n, nq, d, k):
    base = _angular(n, d, 1)
    q = _angular(nq, d, 2)
    ids, dd, rep = gpu_knn(base, q, k, M_COS, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, k, M_COS)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dd, d_o)
    assert rep["precision_used"] == 1
    assert rep["rows_fallback"] <= nq // 50, rep


def test_bf16_cosine_graph_and_unnormalised_rows(gpu_lib, orc):
    rng = np.random.default_rng(5)
    data = _angular(8000, 128, 3) * rng.uniform(0.1, 10.0, size=(8000, 1)).astype(np.float32)
    g, gd = gpu_graph(data, 15, M_COS, precision="bf16")
    g_o, gd_o = orc.knn_graph_f32(data, 15, M_COS)
    assert np.array_equal(g, g_o) and same_bits(gd, gd_o)


def test_bf16_cosine_zero_rows_fall_back(gpu_lib, orc):
    base = _angular(6000, 128, 4)
    base[[5, 777, 4000]] = 0.0
    q = _angular(100, 128, 6)
    q[[3, 50]] = 0.0
    ids, dd, rep = gpu_knn(base, q, 10, M_COS, precision="bf16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 10, M_COS)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dd, d_o)
    assert rep["rows_fallback"] >= 2


def test_bf16_cosine_full_size_equals_fp32_kernel(gpu_lib):
    # N=290,000 angular points (d=256), 10,000 queries, k=20: both GPU forms agree bit for bit
    base = _angular(290000, 256, 1)
    q = _angular(10000, 256, 2)
    i32, d32 = gpu_knn(base, q, 20, M_COS, precision="fp32")
    ib, db, rep = gpu_knn(base, q, 20, M_COS, precision="bf16", report=True)
    assert np.array_equal(i32, ib) and same_bits(d32, db)
    assert rep["rows_fallback"] <= 100, rep


def _fp64_dist(base, q, ids, metric):
    b = base.astype(np.float64)[ids]                  # [nq][k][d]
    x = q.astype(np.float64)[:, None, :]
    if metric == M_COS:
        r = 1.0 - (b * x).sum(-1) / (np.sqrt((b * b).sum(-1)) * np.sqrt((x * x).sum(-1)))
        return np.maximum(r, 0.0)
    s = ((b - x) ** 2).sum(-1)
    return np.sqrt(s) if metric == M_EUC else s


@pytest.mark.parametrize("metric", [M_SQ, M_EUC, M_COS])
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_report_max_fp64_error(gpu_lib, metric, precision):
    # the report's max |returned - FP64| over every returned neighbour
    from manifoldann_gb300 import synthetic

    base = synthetic.iid_normal(6000, 160, seed=41)
    q = synthetic.iid_normal(150, 160, seed=42)
    ids, d, rep = gpu_knn(base, q, 12, metric, precision=precision, report=True, fp64_error=True)
    want = np.abs(d.astype(np.float64) - _fp64_dist(base, q, ids, metric)).max()
    got = rep["max_abs_err_fp64"]
    assert got >= 0.0
    assert abs(got - want) <= 1e-9 * max(1.0, float(np.abs(d).max()))
    # FP32 distances of these sizes stay within a few ulps x d of FP64
    assert got <= 1e-4 * max(1.0, float(np.abs(d).max()))
    _, _, rep0 = gpu_knn(base, q, 12, metric, precision=precision, report=True)
    assert rep0["max_abs_err_fp64"] == -1.0


# ---- the FP8 (e4m3) form: per-row power-of-two scales, the same certificate
# and exact FP32 rerank; its window is wide, so many rows fall back to the
# exact FP32 scan -- the answer is the FP32 oracle's either way

@pytest.mark.parametrize("kind,n,nq,d,k,metric", [("mix", 6000, 300, 256, 10, M_SQ), ("iid", 5000, 200, 128, 10, M_SQ),
                                                 ("iid", 3000, 150, 40, 7, M_EUC), ("ang", 9000, 200, 256, 20, M_COS),
                                                 ("mix", 40000, 300, 784, 10, M_SQ)])
def test_fp8_form_equals_oracle(gpu_lib, orc, kind, n, nq, d, k, metric):
    from manifoldann_gb300 import synthetic

    if kind == "mix":
        base, q = synthetic.quantized_mixture(n, d, seed=11), synthetic.quantized_mixture(nq, d, seed=12)
    elif kind == "ang":
        base, q = _angular(n, d, 11), _angular(nq, d, 12)
    else:
        base, q = synthetic.iid_normal(n, d, seed=11), synthetic.iid_normal(nq, d, seed=12)
    ids, dd, rep = gpu_knn(base, q, k, metric, precision="fp8", report=True)
    ids_o, d_o = orc.knn_f32(base, q, k, metric)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dd, d_o)
    assert rep["precision_used"] == 2
    ids64, _ = gpu_knn(base, q, k, metric, precision="fp8", fp64_ties=True)
    assert np.array_equal(ids64, orc.knn_f64(base, q, k, metric)[0])


def test_fp8_form_graph(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    data = synthetic.quantized_mixture(5000, 128, seed=13)
    g, gd = gpu_graph(data, 12, M_SQ, precision="fp8")
    g_o, gd_o = orc.knn_graph_f32(data, 12, M_SQ)
    assert np.array_equal(g, g_o) and same_bits(gd, gd_o)


# ---- FP16 form (MANN_PREC_FP16): FP16 main columns scaled by a power of two,
# the norm fold as a BF16 step; the same certificate and exact FP32 rerank


@pytest.mark.parametrize("kind,n,nq,d,k,metric", [("ang", 20000, 600, 256, 20, M_COS), ("aniso", 20000, 400, 128, 10, M_SQ),
                                                 ("aniso", 8000, 300, 96, 10, M_EUC), ("iid", 5000, 200, 40, 7, M_SQ),
                                                 ("mix", 6000, 300, 784, 10, M_SQ), ("ang", 9000, 200, 200, 24, M_COS)])
def test_fp16_form_equals_oracle(gpu_lib, orc, kind, n, nq, d, k, metric):
    from manifoldann_gb300 import synthetic

    if kind == "mix":
        base, q = synthetic.quantized_mixture(n, d, seed=21), synthetic.quantized_mixture(nq, d, seed=22)
    elif kind == "ang":
        base, q = _angular(n, d, 21), _angular(nq, d, 22)
    elif kind == "aniso":
        base = synthetic.anisotropic_clusters(n, d, seed=21, clusters=64)
        q = synthetic.anisotropic_clusters(nq, d, seed=22, clusters=64)
    else:
        base, q = synthetic.iid_normal(n, d, seed=21), synthetic.iid_normal(nq, d, seed=22)
    ids, dd, rep = gpu_knn(base, q, k, metric, precision="fp16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, k, metric)
    assert np.array_equal(ids, ids_o)
    assert same_bits(dd, d_o)
    assert rep["precision_used"] == 4
    assert rep["rows_fallback"] <= nq // 50, rep
    ids64, _ = gpu_knn(base, q, k, metric, precision="fp16", fp64_ties=True)
    assert np.array_equal(ids64, orc.knn_f64(base, q, k, metric)[0])


def test_auto_takes_fp16_rows_where_bf16_cannot_hold_the_data(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    for data, q, want in ((synthetic.anisotropic_clusters(6000, 128, seed=31, clusters=16),
                           synthetic.anisotropic_clusters(200, 128, seed=32, clusters=16), 4),
                          (synthetic.quantized_mixture(6000, 256, seed=33), synthetic.quantized_mixture(200, 256, seed=34), 1)):
        ids, dd, rep = gpu_knn(data, q, 10, M_SQ, precision="auto", report=True)
        ids_o, d_o = orc.knn_f32(data, q, 10, M_SQ)
        assert np.array_equal(ids, ids_o) and same_bits(dd, d_o)
        assert rep["precision_used"] == want, rep


def test_fp16_form_graph(gpu_lib, orc):
    from manifoldann_gb300 import synthetic

    data = synthetic.anisotropic_clusters(7000, 64, seed=23, clusters=32)
    g, gd = gpu_graph(data, 12, M_SQ, precision="fp16")
    g_o, gd_o = orc.knn_graph_f32(data, 12, M_SQ)
    assert np.array_equal(g, g_o) and same_bits(gd, gd_o)


@pytest.mark.parametrize("mag", [1e15, 1e-15])
def test_fp16_form_scales_into_range(gpu_lib, orc, mag):
    """Rows far outside FP16's range are scaled by a power of two into it (the
    answers and their distance bits stay the FP32 form's)."""
    from manifoldann_gb300 import synthetic

    base = (synthetic.iid_normal(6000, 64, seed=24) * np.float32(mag)).astype(np.float32)
    q = (synthetic.iid_normal(150, 64, seed=25) * np.float32(mag)).astype(np.float32)
    ids, dd, rep = gpu_knn(base, q, 10, M_SQ, precision="fp16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 10, M_SQ)
    assert np.array_equal(ids, ids_o) and same_bits(dd, d_o)
    assert rep["rows_fallback"] <= 3, rep


def test_fp16_form_outlier_beyond_range_stays_exact(gpu_lib, orc):
    """A point far beyond the sampled range saturates in FP16; its bound makes
    the certificate fail instead of admitting a wrong answer."""
    from manifoldann_gb300 import synthetic

    base = synthetic.iid_normal(5000, 32, seed=26)
    base[4321] *= np.float32(1e6)  # not among the scale probe's rows (every 4th row)
    q = synthetic.iid_normal(100, 32, seed=27)
    q[7] = base[4321] * np.float32(0.999)
    ids, dd, rep = gpu_knn(base, q, 5, M_SQ, precision="fp16", report=True)
    ids_o, d_o = orc.knn_f32(base, q, 5, M_SQ)
    assert np.array_equal(ids, ids_o) and same_bits(dd, d_o)


def test_fp64_tie_order_at_the_bit_level(gpu_lib, orc):
    """Squared distances from the origin that FP32 cannot tell apart (all round
    to 1 + 2^-22) but FP64 can: gaps of 2^-30 and 2^-32 (ordered by the
    double-float values alone), 2^-46 (inside their error window: FP64
    sequential sums decide) and an exact tie (ids decide).  Lower ids sit on
    the larger distances, so FP32 (distance, id) order differs from the
    oracle's at every position of the cluster."""
    d = 8
    pts = np.zeros((5, d), np.float32)
    pts[0, 0] = np.float32(1.0 + 2.0 ** -23)                    # 1 + 2^-22 + 2^-46
    pts[1, :3] = [1.0, 2.0 ** -11, 2.0 ** -15]                  # 1 + 2^-22 + 2^-30
    pts[2, :4] = [1.0, 2.0 ** -11, 0.0, 2.0 ** -16]             # 1 + 2^-22 + 2^-32
    pts[3, :5] = [1.0, 2.0 ** -11, 0.0, 0.0, 2.0 ** -23]        # 1 + 2^-22 + 2^-46 (ties id 0)
    pts[4, :2] = [1.0, 2.0 ** -11]                              # 1 + 2^-22
    rng = np.random.default_rng(21)
    inner = (rng.standard_normal((4, d)) * 0.2).astype(np.float32)
    far = (rng.standard_normal((3000, d)) * 0.3 + 3.0).astype(np.float32)
    base = np.concatenate([pts, far, inner])
    q = np.zeros((4, d), np.float32)
    for metric in (M_SQ, M_EUC):
        ids_o, _ = orc.knn_f64(base, q, 9, metric)
        assert list(ids_o[0, 4:9]) == [4, 0, 3, 2, 1]
        for precision in ("fp32", "bf16"):
            ids64, _, rep = gpu_knn(base, q, 9, metric, precision=precision, fp64_ties=True, report=True)
            assert np.array_equal(ids64, ids_o), (precision, metric, ids64[0], ids_o[0])
            assert rep["rows_unresolved"] == 0, rep
