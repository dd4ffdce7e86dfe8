"""The oracle's restatements of src/mul.jl and of the Gram product
(src/scaling.jl:274-296) against dense linear algebra."""
import numpy as np
import scipy.sparse as sp

from oracle import severo_oracle as O


def test_mul_spvec_and_sparse_match_dense():
    rng = np.random.default_rng(1)
    A = sp.random(40, 30, density=0.2, random_state=2, format="csc")
    x = sp.random(30, 1, density=0.3, random_state=3, format="csc")
    y0 = rng.standard_normal(40)
    y = O.mul_spvec(A, x.indices, x.data, 2.0, 0.5, y0)
    assert np.allclose(y, 2.0 * (A @ x.toarray().ravel()) + 0.5 * y0, rtol=1e-13, atol=1e-13)
    assert np.array_equal(O.mul_spvec(A, x.indices, x.data, 0.0, 0.0, y0), np.zeros(40))
    B = sp.random(30, 12, density=0.25, random_state=4, format="csc")
    C0 = rng.standard_normal((40, 12))
    C = O.mul_sparse(A, B, 1.5, 2.0, C0)
    assert np.allclose(C, 1.5 * (A @ B).toarray() + 2.0 * C0, rtol=1e-13, atol=1e-13)


def test_gram_matches_dense():
    X = O.synth_counts(300, 80, -0.5, 1.5, depth=0.8, seed=5)
    Xn = O.normalize_cells(X, "lognormalize", 1e4, np.float64)
    S1, _, _ = O.scale_features(Xn, 10.0, np.float64, np.arange(1, 41))
    S2, _, _ = O.scale_features(Xn, 10.0, np.float64, np.arange(30, 71))
    for Sl, Sr in ((S1, S1), (S1, S2)):
        G = O.gram(Sl, Sr, 2.0)
        assert np.allclose(G, 2.0 * Sl.dense().T @ Sr.dense(), rtol=1e-12, atol=1e-10)
