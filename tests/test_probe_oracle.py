"""The probe oracle's own gradient against central finite differences (FP64,
no BF16 rounding): the oracle is the definition of the learned probe, and this
pins it (no GPU)."""
import numpy as np
import pytest


@pytest.mark.parametrize("prior", [False, True])
def test_oracle_gradient_matches_finite_differences(prior):
    from oracle import probe as P

    rng = np.random.default_rng(1 + prior)
    dims = (5, 7, 6, 9)
    n = P.layout(*dims)["total"]
    params = rng.standard_normal(n) * 0.5
    params[-1] = np.log(0.3)
    X = rng.standard_normal((11, dims[0]))
    labels = rng.integers(-1, dims[3], size=(11, 4)).astype(np.int32)
    C = rng.standard_normal((dims[3], dims[0])) if prior else None
    loss, g = P.forward_backward(params, dims, X, labels, C, bf16_round=False)
    h = 1e-6
    idx = rng.choice(n, 60, replace=False)
    if prior:
        idx = np.append(idx, n - 1)
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        lp, _ = P.forward_backward(params + e, dims, X, labels, C, bf16_round=False)
        lm, _ = P.forward_backward(params - e, dims, X, labels, C, bf16_round=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
    if not prior:
        assert g[-1] == 0.0


def test_bf16_rounding_ties_to_even():
    from oracle import probe as P

    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-8, 1.0 + 2**-9, -2.5, 3.0e38], np.float32)
    r = P.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2**-6 and r[3] == 1.0
    assert r[4] == -2.5
