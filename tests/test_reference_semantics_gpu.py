"""Where the GPU's IVF routing and KMeans assignment can differ from the
reference's arithmetic, and by how much.

The reference routes an IVF query by GEMV-form centroid distances
||c||^2 + ||q||^2 - 2 c.q in FP32 (src/indices/ivf_flat.jl:103-131) and
partialsortperm (:150), and assigns KMeans clusters by GEMM-form distances and
a strict-< arg-min (src/transforms/kmeans/distance.jl:68-107,287-310).  The
GPU routes by the exact FP32 difference-form distances and assigns by the
exact arg-min (near-ties ordered in FP64).  Both are roundings of the same
exact distances, so they can only disagree where two centroids' exact
distances lie within the GEMV/GEMM form's FP32 error of each other.  These
tests measure the agreement on a slice of the 1M x 128 workload (200,000
points, 1,024 lists) and assert that every disagreement is such a near-tie;
where the probed lists agree, the search results are identical to the
reference's IVF-Flat query (bounded max-heap, strict-< admission).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def _gemv_err(cn, qn, d):
    """Bound of |fl(||c||^2 + ||q||^2 - 2 c.q) - exact| for sequential FP32
    sums of d terms: each of the three sums carries gamma_d = d u / (1 - d u)
    of its magnitude (|c.q| <= ||c|| ||q||), plus the two final roundings."""
    g = d * U / (1.0 - d * U)
    mag = cn + qn + 2.0 * np.sqrt(cn * qn)
    return 2.0 * (g * mag + 2.0 * U * (cn + qn))


@pytest.fixture(scope="module")
def slice_set():
    import manifoldann_gb300 as M
    from manifoldann_gb300 import synthetic

    X = synthetic.anisotropic_clusters(200_000, 128, seed=1, clusters=256)
    Q = synthetic.anisotropic_clusters(2000, 128, seed=3, clusters=256)
    idx = M.build_index(M.IVFFlatIndex, X.T, nlist=1024, distance=M.SqEuclidean(), seed=1)
    return X, Q, idx


def test_ivf_routing_and_search_vs_reference_semantics(gpu_lib, orc, slice_set):
    X, Q, idx = slice_set
    d = X.shape[1]
    C = np.ascontiguousarray(idx.centroids.T, dtype=np.float32)
    cn = orc.centroid_norms_f32(C)
    npb, k = 8, 10
    ids_g, d_g = idx.search_arrays(X.T, Q.T, k, nprobe=npb)
    ids_r, d_r = orc.ivf_query_f32(X, C, cn, idx.list_offsets, idx.list_ids, Q, k, npb, orc.SQEUCLIDEAN,
                                   orc.EUCLIDEAN)
    p_ref = orc.ivf_route_gemv_f32(C, cn, Q, npb, orc.EUCLIDEAN)
    p_gpu, _ = orc.knn_f32(C, Q, npb, orc.EUCLIDEAN)  # the GPU's routing: exact FP32 top-nprobe
    C64, Q64 = C.astype(np.float64), Q.astype(np.float64)
    cn64 = (C64 * C64).sum(1)
    same_probes = np.array([set(a) == set(b) for a, b in zip(p_ref, p_gpu)])
    for i in np.nonzero(~same_probes)[0]:
        q = Q64[i]
        D = ((C64 - q) ** 2).sum(1)
        err = _gemv_err(cn64, float(q @ q), d) + 4.0 * U * D  # + the exact form's and sqrt's roundings
        ref_only = np.array(sorted(set(p_ref[i]) - set(p_gpu[i])))
        gpu_only = np.array(sorted(set(p_gpu[i]) - set(p_ref[i])))
        gap = np.abs(D[ref_only][:, None] - D[gpu_only][None, :])
        slack = err[ref_only][:, None] + err[gpu_only][None, :]
        assert (gap <= slack).all(), (i, gap.max(), slack.min())
    # identical probed lists: identical answers (ids and distance bits)
    same_ids = (ids_g == ids_r).all(1)
    same_bits = (d_g.view(np.uint32) == d_r.view(np.uint32)).all(1)
    assert (same_ids & same_bits)[same_probes].all()
    rate_probes = float(same_probes.mean())
    rate_results = float((same_ids & same_bits).mean())
    print(f"\nIVF routing agreement with the GEMV form: {rate_probes:.4f} of queries; "
          f"identical results: {rate_results:.4f}")
    assert rate_probes >= 0.99 and rate_results >= 0.99


def test_kmeans_assign_vs_reference_gemm_form(gpu_lib, orc, slice_set):
    import manifoldann_gb300 as M

    X, _, idx = slice_set
    d = X.shape[1]
    C = np.ascontiguousarray(idx.centroids.T, dtype=np.float32)
    for metric, mobj in ((orc.EUCLIDEAN, M.Euclidean()), (orc.SQEUCLIDEAN, M.SqEuclidean())):
        a_g, _ = M.assign_arrays(X.T, idx.centroids, mobj)
        a_r, _ = orc.kmeans_assign_gemm_f32(X, C, metric)
        diff = np.nonzero(a_g != a_r)[0]
        C64 = C.astype(np.float64)
        for j in diff:
            x = X[j].astype(np.float64)
            Da = float(((C64[a_g[j]] - x) ** 2).sum())
            Db = float(((C64[a_r[j]] - x) ** 2).sum())
            xn = float(x @ x)
            ea = _gemv_err(float(C64[a_g[j]] @ C64[a_g[j]]), xn, d) + 4.0 * U * Da
            eb = _gemv_err(float(C64[a_r[j]] @ C64[a_r[j]]), xn, d) + 4.0 * U * Db
            assert Da <= Db + 1e-12 * max(Da, 1.0)  # the GPU's pick is the exact arg-min
            assert Db - Da <= ea + eb, (j, Db - Da, ea + eb)
        rate = 1.0 - len(diff) / len(X)
        print(f"\nKMeans assignment agreement with the GEMM form (metric {metric}): {rate:.6f} "
              f"({len(diff)} of {len(X)} points differ, each a near-tie)")
        assert rate >= 0.999
