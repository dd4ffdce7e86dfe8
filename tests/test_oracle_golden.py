"""Pins the CPU oracle against the literal fixtures of Severo.jl's own tests
(tests/golden/golden.json, written by tests/golden/make_golden.py) and against the
properties those tests assert.  CPU only."""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import severo_oracle as O

G = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())


def test_normalize_relativecounts_golden():
    # test/test_input.jl:62-74
    C = sp.csc_matrix(np.array(G["normalize"]["counts"]))
    Q = O.normalize_cells(C, "relativecounts")
    assert Q.dtype == np.float64
    assert np.allclose(Q.toarray(), G["normalize"]["relative"], rtol=1e-15, atol=0)
    assert np.allclose(Q.sum(axis=1), 1.0)
    Q10 = O.normalize_cells(C, "relativecounts", scale_factor=10.0)
    assert np.allclose(Q10.toarray(), G["normalize"]["relative_sf10"], rtol=1e-15)
    assert np.allclose(Q10.sum(axis=1), 10.0)


def test_normalize_log_golden():
    C = sp.csc_matrix(np.array(G["normalize"]["counts"]))
    Q2 = O.normalize_cells(C, "lognormalize")
    assert np.allclose(Q2.toarray(), G["normalize"]["log"], rtol=1e-15)


def test_normalize_float32_and_unknown_method():
    C = sp.csc_matrix(np.array(G["normalize"]["counts"]))
    assert O.normalize_cells(C, "relativecounts", dtype=np.float32).dtype == np.float32
    assert O.normalize_cells(C, "lognormalize", dtype=np.float32).dtype == np.float32
    with pytest.raises(ValueError):
        O.normalize_cells(C, "bogus")


def test_scaling_golden():
    # test/test_scaling.jl:21-45
    X = sp.csc_matrix(np.array(G["scaling"]["counts"]))
    S, mean, std = O.scale_features(X.astype(np.float64))
    assert np.allclose(mean, G["scaling"]["mean"], rtol=1e-14)
    assert np.allclose(std, G["scaling"]["std"], rtol=1e-14)
    assert np.allclose(S.mu, G["scaling"]["mu"], rtol=1e-14)
    assert np.allclose(S.dense(), G["scaling"]["dense"], rtol=1e-13, atol=1e-14)


def test_mean_var_welford_matches_vectorised():
    X = sp.csc_matrix(np.array(G["scaling"]["counts"]))
    mean, var = O.mean_var(X)
    for j in range(X.shape[1]):
        col = X[:, j]
        m, v = O.mean_var_column(col.data, X.shape[0])
        assert abs(m - mean[j]) < 1e-14 and abs(v - var[j]) < 1e-13


def test_float32_accumulation_follows_the_reference():
    """For Float32 data the reference accumulates the moments in Float32
    (src/scaling.jl:40-44); the oracle's default does the same, column by
    column as mean_var_column, while acc=Float64 (the device's choice) gives
    the FP64 moments of the same values."""
    X = O.synth_counts(1500, 200, -1.0, 1.5, depth=0.5, seed=41)
    Xn = O.normalize_cells(X, "lognormalize", 1e4, np.float32)
    m32, v32 = O.mean_var_welford(Xn, np.float32)
    for j in (0, 7, 123):
        col = Xn[:, j]
        m, v = O.mean_var_column(col.data, Xn.shape[0], acc=np.float32)
        assert m == m32[j] and v == v32[j]
    _, mean_ref, std_ref = O.scale_features(Xn, 10.0, np.float32)            # reference: Float32
    _, mean_64, std_64 = O.scale_features(Xn, 10.0, np.float32, acc=np.float64)
    assert std_ref.dtype == np.float32
    m64, v64 = O.mean_var(Xn)
    assert np.array_equal(std_ref, np.sqrt(v32).astype(np.float32))
    assert np.array_equal(std_64, np.sqrt(v64.astype(np.float32)))
    # the two differ by Float32 rounding of the running sums only
    assert np.allclose(std_ref, std_64, rtol=2e-5)


def test_scale_clip_upper_only():
    # scaling.jl:209-212: upper clip only; zeros never clipped
    X = sp.csc_matrix(np.array(G["scaling"]["counts"], dtype=np.float64))
    S, mean, std = O.scale_features(X, scale_max=0.5)
    D = S.dense()
    assert D.max() <= 0.5 + 1e-12
    Z = X.toarray() == 0
    assert np.allclose(D[Z], -np.broadcast_to(S.mu, D.shape)[Z])


@pytest.mark.parametrize("variant", ["dense", "sparse"])
def test_centered_matrix_golden(variant):
    # test/test_scaling.jl:70-113
    c = G["centered"]
    A = np.array(c["A"])
    Cm = O.CenteredMatrix(sp.csc_matrix(A) if variant == "sparse" else A, np.array(c["mu"]))
    r = np.array(c["r"])
    y0 = np.array(c["y0"])
    e = c[variant]
    assert np.allclose(Cm.mul(r), e["Cr"], rtol=1e-14)
    y = Cm.mul(r, 2.0, 1.0, y0)
    assert np.allclose(y, e["y1"], rtol=1e-14)
    if variant == "sparse":
        y = Cm.mul(r, 2.0, 1.0, y)
        assert np.allclose(y, e["y2"], rtol=1e-14)
    assert np.allclose(Cm.rmul(y), e["Cty"], rtol=1e-14)
    assert np.allclose(Cm.rmul(y, 2.0, 1.0, r), e["r1"], rtol=1e-14)


def test_mean_var_grouped_golden():
    g = G["mean_var_grouped"]
    for case in g["cases"]:
        mu, var, n = O.mean_var_grouped(g["idx"], g["val"], g["n"], case["labels"], case["nlabels"])
        assert np.allclose(mu, case["mu"], rtol=1e-13)
        assert np.allclose(var, case["var"], rtol=1e-12)
        assert list(n) == case["n"]


@pytest.mark.parametrize("case", range(3))
def test_snn_golden(case):
    s = G["snn"]
    nn = np.array(s["nn_index"])
    c = s["cases"][case]
    Gr = O.knn_graph(nn, nn.shape[0])
    W = O.jaccard_index(Gr, s["k"], c["prune"])
    E = sp.csc_matrix((c["vals"], (np.array(c["rows"]) - 1, np.array(c["cols"]) - 1)), shape=W.shape)
    E.sort_indices()
    assert np.array_equal(W.indptr, E.indptr) and np.array_equal(W.indices, E.indices)
    assert np.array_equal(W.data, E.data)        # bit-exact


def test_snn_diag_variant_equals_k_variant_for_regular_graphs():
    s = G["snn"]
    nn = np.array(s["nn_index"])
    Gr = O.knn_graph(nn, nn.shape[0])
    a = O.jaccard_index(Gr, s["k"], 1 / 15)
    b = O.jaccard_index(Gr, None, 1 / 15)
    assert (a != b).nnz == 0


@pytest.mark.parametrize("shape,nu,tol", [((50, 50), 20, 1e-5), ((100, 50), 20, 1e-5)])
def test_irlba_dense(shape, nu, tol):
    # test/test_irlba.jl:25-41
    rng = np.random.default_rng(3)
    X = rng.standard_normal(shape)
    U, s, V, info, it, nmv = O.irlba(lambda x: X @ x, lambda y: X.T @ y, *shape, nu, tol=tol,
                                     rng=rng)
    ss = np.linalg.svd(X, compute_uv=False)
    assert info == 0
    assert np.linalg.norm(s - ss[:nu]) <= 1.5e-8 * np.linalg.norm(ss[:nu])
    assert np.linalg.norm(X.T @ U - V * s) / np.linalg.norm(X) < tol


def test_irlba_centered_sparse():
    # test/test_irlba.jl:79-91
    X = sp.random(2000, 400, density=0.1, random_state=5, format="csc")
    mu = np.asarray(X.mean(axis=0)).ravel()
    Cm = O.CenteredMatrix(X, mu)
    U, s, V, info, _, _ = O.irlba(Cm.mul, Cm.rmul, 2000, 400, 2, tol=1e-9)
    Q = Cm.dense()
    ss = np.linalg.svd(Q, compute_uv=False)
    assert info == 0
    assert np.allclose(s, ss[:2], rtol=1e-10)
    assert np.linalg.norm(Q.T @ U - V * s) / np.linalg.norm(Q) < 1e-9


def test_knn_exact_matches_pairwise():
    # test/test_nn.jl:23-39 brute force
    rng = np.random.default_rng(0)
    X = rng.random((100, 10))
    idx, dist = O.knn_exact(X, 4)
    D = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    for i in range(100):
        ref = np.argsort(D[i], kind="stable")[:4]
        assert set(ref) == set(idx[i])
        assert idx[i, 0] == i
        assert np.allclose(dist[i], np.sort(D[i])[:4])


def test_knn_exact_cosine_and_exclude_self():
    rng = np.random.default_rng(1)
    X = rng.random((80, 6))
    idx, dist = O.knn_exact(X, 5, include_self=False, metric="cosine")
    Xn = X / np.linalg.norm(X, axis=1, keepdims=True)
    D = 1 - Xn @ Xn.T
    np.fill_diagonal(D, np.inf)
    for i in range(80):
        assert i not in idx[i]
        assert set(np.argsort(D[i], kind="stable")[:5]) == set(idx[i])


def test_round_bf16():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float32)
    r = O.round_bf16(x)
    # values representable in bf16 are unchanged; ties round to even
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert r[3] == -2.5
