"""TopKRouting / select_indices host mirror against the reference's routing
known answers and the oracle's top-k routing (no GPU)."""
import numpy as np
import pytest


def test_select_indices_known_answers():
    # test/unit/indices/multilevel/routing_tests.jl:8-56
    import manifoldann_gb300 as M

    d = np.array([0.9, 0.8, 0.7, 0.6, 0.5, 0.1, 0.2], np.float32)
    assert M.select_indices(M.TopKRouting(3), d, 5) == [5, 4, 3]
    assert M.select_indices(M.TopKRouting(10), np.array([0.4, 0.3, 0.2, 0.1], np.float32), 4) == [4, 3, 2, 1]
    assert M.select_indices(M.TopKRouting(3), np.array([0.1, 0.2], np.float32), []) == []
    with pytest.raises(M.ArgumentError):
        M.select_indices(M.TopKRouting(5), np.array([], np.float32), 3)
    with pytest.raises(M.ArgumentError):
        M.TopKRouting(0)


def test_select_indices_matches_oracle(orc):
    import manifoldann_gb300 as M

    rng = np.random.default_rng(3)
    for trial in range(200):
        n = int(rng.integers(1, 60))
        d = rng.choice(np.array([0.0, -0.0, 1.0, 2.0, np.nan, np.inf], np.float32), n) \
            if trial % 3 == 0 else rng.standard_normal(n).astype(np.float32)
        nc = int(rng.integers(1, 70))
        k = int(rng.integers(1, 20))
        got = M.select_indices(M.TopKRouting(k), d, nc)
        assert got == (orc.topk_route(d, nc, k) + 1).tolist()
