"""The multi-threaded CPU restatement (oracle/cpu_path.c, the CPU baseline and
the reference arm of bench.py) against the numpy oracle: the same arithmetic,
so the same numbers, whatever the thread count."""
import numpy as np
import pytest

from oracle import cpu_path as CP
from oracle import severo_oracle as O


@pytest.fixture(scope="module")
def counts():
    rng = np.random.default_rng(4)
    mu_g = rng.lognormal(-1.0, 1.5, 600)
    s_c = rng.lognormal(0.0, 0.3, 400)
    return CP.generate(400, 600, mu_g, s_c, depth=0.5, dispersion=0.2, seed=9, nt=3), mu_g, s_c


def test_generator_is_seeded_and_thread_independent(counts):
    X, mu_g, s_c = counts
    Y = CP.generate(400, 600, mu_g, s_c, depth=0.5, dispersion=0.2, seed=9, nt=1)
    assert (X != Y).nnz == 0 and np.array_equal(X.indptr, Y.indptr)
    X.has_sorted_indices = False
    assert np.array_equal(X.sorted_indices().indices, Y.indices)
    # NB(mean m, size 5): E[x] = m; the sample mean of all counts is close to it
    expect = 0.5 * np.outer(s_c, mu_g).sum()
    assert abs(X.sum() - expect) < 0.05 * expect


def test_normalize_and_scale_match_oracle(counts):
    X = counts[0]
    Xn, tot = CP.normalize(X, 1e4, True, nt=4)
    ref = O.normalize_cells(X, "lognormalize", 1e4, np.float64)
    assert np.array_equal(tot, np.asarray(X.sum(axis=1)).ravel())
    assert np.allclose(Xn.data, ref.data, rtol=1e-15, atol=0)
    feats = O.top_variable_genes(ref, 120)
    S, mean, std = CP.scale(Xn, feats, 10.0, nt=4)
    Sr, rmean, rstd = O.scale_features(ref, 10.0, np.float64, feats)
    assert np.allclose(mean, rmean, rtol=1e-13) and np.allclose(std, rstd, rtol=1e-13)
    assert np.allclose(S.mu, Sr.mu, rtol=1e-13)
    assert np.allclose(S.val, Sr.A.data, rtol=1e-13)
    x = np.random.default_rng(1).standard_normal(S.n)
    u = np.random.default_rng(2).standard_normal(S.m)
    assert np.allclose(S.mul(x), Sr.mul(x), rtol=1e-12, atol=1e-12)
    assert np.allclose(S.rmul(u), Sr.rmul(u), rtol=1e-12, atol=1e-12)


def test_pipeline_singular_values_and_neighbours(counts):
    X = counts[0]
    ref = O.normalize_cells(X, "lognormalize", 1e4, np.float64)
    feats = O.top_variable_genes(ref, 120)
    t, Z, info = CP.pipeline(X, feats, npcs=10, k=8, tol=1e-9, nt=2)
    assert set(t) == {"normalize", "scale", "pca", "knn"}
    Sr, _, _ = O.scale_features(ref, 10.0, np.float64, feats)
    sf = np.linalg.svd(Sr.dense(), compute_uv=False)[:10]
    assert np.max(np.abs(info["sigma"] - sf) / sf) < 1e-8
    idx = CP.knn(Z, 8, nt=2)
    ridx, _ = O.knn_exact(Z, 8)
    assert all(set(a) == set(b) for a, b in zip(idx, ridx))


def test_approximate_search_recall():
    """The random-projection forest of the CPU baseline finds the exact
    neighbours on well-separated mixture data."""
    rng = np.random.default_rng(6)
    n, d = 3000, 20
    X = rng.normal(0, 4, (15, d))[rng.integers(0, 15, n)] + rng.standard_normal((n, d))
    idx = CP.ann(X, 10, nt=2)
    assert np.all(idx[:, 0] == np.arange(n))
    assert CP.recall(X, idx, 10, np.arange(0, n, 7)) > 0.99
