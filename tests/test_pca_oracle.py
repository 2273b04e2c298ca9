"""Local PCA: the FP64 oracle on the reference's own PCA test cases
(test/unit/geometry/pca_tests.jl) and the PCAMethod argument checks (no GPU)."""
import numpy as np
import pytest


def test_pca_method_validation():
    # pca_tests.jl:6-38
    import manifoldann_gb300 as M

    m = M.PCAMethod()
    assert m.intrinsic_dim is None and m.min_variance_ratio == 0.95
    assert M.PCAMethod(intrinsic_dim=3, min_variance_ratio=0.8).intrinsic_dim == 3
    for kw in ({"intrinsic_dim": 0}, {"intrinsic_dim": -1}, {"min_variance_ratio": 0.0},
               {"min_variance_ratio": 1.5}, {"min_variance_ratio": -0.1}):
        with pytest.raises(M.ArgumentError):
            M.PCAMethod(**kw)


def test_oracle_reference_cases():
    from oracle import pca

    rng = np.random.default_rng(42)
    # 2-D plane in 3-D (pca_tests.jl:56-73): two dimensions, the plane's normal is orthogonal to the basis
    xy = rng.standard_normal((2, 30))
    data = np.vstack([xy, 0.5 * xy[0] + 0.3 * xy[1]]).T
    dim, vals, basis = pca.fit_pca(data[0], data[1:], intrinsic_dim=2)
    normal = np.array([0.5, 0.3, -1.0]) / np.linalg.norm([0.5, 0.3, -1.0])
    assert dim == 2 and basis.shape == (3, 2) and np.abs(basis.T @ normal).max() < 1e-10
    # 1-D line (pca_tests.jl:75-92): alignment > 0.99
    t = rng.standard_normal(20)
    direction = np.array([1.0, 2.0, 3.0]) / np.linalg.norm([1.0, 2.0, 3.0])
    data = np.outer(t, direction)
    dim, vals, basis = pca.fit_pca(data[0], data[1:], intrinsic_dim=1)
    assert abs(basis[:, 0] @ direction) > 0.99
    # auto dimension (pca_tests.jl:94-108)
    data = np.vstack([rng.standard_normal((2, 50)) * 10, rng.standard_normal((1, 50)) * 0.01]).T
    dim, _, _ = pca.fit_pca(data[0], data[1:], min_variance_ratio=0.99)
    assert dim == 2
    # the dual (d > k) path gives orthonormal directions too
    nb = rng.standard_normal((6, 40))
    dim, vals, basis = pca.fit_pca(np.zeros(40), nb, intrinsic_dim=4)
    assert np.allclose(basis.T @ basis, np.eye(4), atol=1e-10)
