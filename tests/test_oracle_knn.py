"""The oracle's sampled-query kNN agrees with its full brute force."""
import numpy as np
import pytest


@pytest.mark.parametrize("include_self", [True, False])
def test_knn_exact_queries_matches_full(O, include_self):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((6000, 12))
    q = rng.choice(6000, 40, replace=False)
    full, _ = O.knn_exact(X, 10, include_self)
    part = O.knn_exact_queries(X, q, 10, include_self, block=1000)
    assert np.array_equal(full[q], part)
